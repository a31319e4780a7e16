"""The index scheme of fft512_cols_kernel (csrc/fft_lines.cu) restated in
numpy: the three radix-8 stages with their twiddles, the task -> (column,
index) mapping and the shared-memory addresses (odd column pitch), checked
against numpy's inverse FFT (times 512), and the addresses checked to stay
inside one buffer and to hit 16 distinct bank pairs per half warp."""
import numpy as np

N, C, PITCH, THREADS = 512, 16, 513, 512
R = C * N // 8 // THREADS
TW = np.exp(2j * np.pi * np.arange(N) / N)


def idft8(a):
    """a[k] <- sum_n a[n] e^{+2 pi i n k / 8}, the kernel's butterfly order."""
    b0, b1 = a[0] + a[4], a[0] - a[4]
    b2, b3 = a[2] + a[6], a[2] - a[6]
    b4, b5 = a[1] + a[5], a[1] - a[5]
    b6, b7 = a[3] + a[7], a[3] - a[7]
    e = [b0 + b2, b1 + 1j * b3, b0 - b2, b1 - 1j * b3]
    o = [b4 + b6, b5 + 1j * b7, b4 - b6, b5 - 1j * b7]
    w = [1.0, (1 + 1j) / np.sqrt(2), 1j, (-1 + 1j) / np.sqrt(2)]
    return [e[k] + w[k] * o[k] for k in range(4)] + [e[k] - w[k] * o[k] for k in range(4)]


def tasks():
    for tid in range(THREADS):
        for r in range(R):
            i = tid + THREADS * r
            yield tid, i % C, i // C


def kernel_tile(x):
    """x: [512 rows][16 columns] complex -> the tile the kernel writes back."""
    sm = np.zeros(C * PITCH, complex)
    for _, c, n1 in tasks():  # stage 1
        v = idft8([x[n1 + 64 * n2, c] for n2 in range(8)])
        for k2 in range(8):
            sm[c * PITCH + n1 * 8 + k2] = v[k2] * TW[n1 * k2]
    regs = {}
    for _, c, rest in tasks():  # stage 2 reads, then (after a barrier) writes
        k2, m1 = rest & 7, rest >> 3
        regs[(c, rest)] = [sm[c * PITCH + m1 * 8 + k2 + 64 * m2] for m2 in range(8)]
    for _, c, rest in tasks():
        k2, m1 = rest & 7, rest >> 3
        v = idft8(regs[(c, rest)])
        for q2 in range(8):
            sm[c * PITCH + k2 * 64 + m1 * 8 + q2] = v[q2] * TW[8 * m1 * q2]
    out = np.zeros_like(x)
    for _, c, rest in tasks():  # stage 3
        k2, q2 = rest & 7, rest >> 3
        v = idft8([sm[c * PITCH + k2 * 64 + q2 + 8 * m1] for m1 in range(8)])
        for q1 in range(8):
            out[k2 + 8 * q2 + 64 * q1, c] = v[q1]
    return out


def test_three_stages_are_the_inverse_dft():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((N, C)) + 1j * rng.standard_normal((N, C))
    got = kernel_tile(x)
    ref = np.fft.ifft(x, axis=0) * N
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_shared_addresses_in_bounds_and_conflict_free():
    # every stage's shared-memory address for the 16 lanes of a half warp
    # (same row or index, columns 0..15): inside the buffer and on 16
    # distinct 8-byte bank pairs (address mod 16 in float2 units)
    def check(addr_of):
        for half in range(THREADS * R // 16):
            i0 = half * 16
            addrs = [addr_of(i % C, i // C) for i in range(i0, i0 + 16)]
            assert max(addrs) < C * PITCH and min(addrs) >= 0
            assert len({a % 16 for a in addrs}) == 16

    for n2 in range(8):
        check(lambda c, n1, n2=n2: c * PITCH + n1 * 8 + n2)               # stage 1 writes (per k2)
        check(lambda c, r, m2=n2: c * PITCH + (r >> 3) * 8 + (r & 7) + 64 * m2)  # stage 2 reads
        check(lambda c, r, q2=n2: c * PITCH + (r & 7) * 64 + (r >> 3) * 8 + q2)  # stage 2 writes
        check(lambda c, r, m1=n2: c * PITCH + (r & 7) * 64 + (r >> 3) + 8 * m1)  # stage 3 reads
    # the row-major landing buffer: stage 1 reads row n1 + 64 n2 of 16 columns
    for n2 in range(8):
        for n1 in range(64):
            addrs = [(n1 + 64 * n2) * C + c for c in range(C)]
            assert len({a % 16 for a in addrs}) == 16 and max(addrs) < N * C <= C * PITCH
