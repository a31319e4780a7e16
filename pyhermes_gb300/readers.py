"""Particle catalogue readers for ``SFCProjection`` (``fin.path``).

Mirrors pyhermes/io/readers.py: the same formats, reader parameters and
output contract -- a dict with ``pos`` (float32 [N, 3], C-contiguous),
``size`` (N) and per-particle fields -- so a parameter file that names a
catalogue on disk works unchanged:

* ``bin``          raw table of ``ncols`` values of ``dtype`` per particle,
                   positions from ``pos_cols``, ``fields`` name other columns;
* ``npz``          NumPy archive, positions under ``pos_key``, every other
                   array (or the ``fields`` mapping) as fields;
* ``gadget``       legacy Gadget format-1 snapshot (Fortran-style records),
                   dark-matter type ``ptype``, split files ``name.0, name.1,
                   ...``: pos, vel, vel_x/y/z and mass per particle;
* ``gadget_hdf5``  Gadget HDF5 snapshot(s), ``PartType{ptype}`` datasets,
                   optional unit scales (needs h5py);
* ``gadget-fof``   legacy Gadget FoF group catalogue (FoF without SUBFIND):
                   group pos, vel, mass;
* ``fof``          Quijote / Pylians ``group_tab_NNN.M`` files (a file, or a
                   catalogue directory with ``snapnum``): positions kpc/h ->
                   Mpc/h, peculiar velocities x (1 + z), masses x 1e10, plus
                   npart and group_offset.

The format is taken from ``fin.format`` or inferred from the file name
(``group_tab_NNN.M`` -> fof, else the suffix).  Remote (http/https) paths
need network access to fetch and are refused with an error.
"""

import os
import re
from pathlib import Path

import numpy as np

_REMOTE = re.compile(r"^[a-zA-Z][a-zA-Z0-9+.-]*://")


def _is_remote(path):
    return bool(_REMOTE.match(str(path))) and not str(path).startswith("file://")


def infer_format(path):
    """Format from the file name (io/readers.py:39-54)."""
    name = Path(str(path)).name
    if re.fullmatch(r"group_tab_\d+\.\d+", name):
        return "fof"
    return {"bin": "bin", "npz": "npz", "gadget": "gadget", "fof": "fof"}.get(Path(name).suffix.lower().lstrip("."))


def _columns(value):
    return [int(v) for v in value] if isinstance(value, (list, tuple, np.ndarray)) else int(value)


def _finish(data, reader):
    """The shared output contract: float32 (N, 3) positions and a size."""
    if not isinstance(data, dict) or "pos" not in data:
        raise ValueError(f"{reader} output must be a dict with a 'pos' array.")
    pos = np.asarray(data["pos"])
    if pos.ndim != 2 or pos.shape[1] != 3:
        raise ValueError(f"{reader} output 'pos' must have shape (N, 3), got {pos.shape}.")
    data["pos"] = np.ascontiguousarray(pos, dtype=np.float32)
    data["size"] = int(data.get("size", pos.shape[0]))
    if data["size"] != pos.shape[0]:
        raise ValueError(f"{reader} output 'size'={data['size']} does not match pos length {pos.shape[0]}.")
    return data


def _with_velocity_components(data):
    vel = data.get("vel")
    if vel is not None:
        vel = np.asarray(vel)
        if vel.ndim == 2 and vel.shape[1] == 3:
            data["vel_x"], data["vel_y"], data["vel_z"] = vel[:, 0], vel[:, 1], vel[:, 2]
    return data


def read_bin(path, dtype="float32", ncols=3, pos_cols=(0, 1, 2), fields=None, **kwargs):
    ncols = int(ncols)
    if ncols <= 0:
        raise ValueError("read_bin requires ncols > 0.")
    raw = np.fromfile(path, dtype=np.dtype(dtype))
    if raw.size % ncols:
        raise ValueError(f"Binary file '{path}' contains {raw.size} values, which cannot be reshaped into "
                         f"(-1, {ncols}).")
    table = raw.reshape(-1, ncols)
    cols = _columns(pos_cols)
    if not isinstance(cols, list) or len(cols) != 3:
        raise ValueError("read_bin requires pos_cols to contain exactly three column indices.")
    data = {"pos": table[:, cols], "size": table.shape[0]}
    for key, sel in (fields or {}).items():
        data[key] = table[:, _columns(sel)]
    return _finish(data, "read_bin")


def read_npz(path, pos_key="pos", fields=None, **kwargs):
    with np.load(path) as z:
        if pos_key not in z:
            raise ValueError(f"NPZ file '{path}' does not contain pos_key='{pos_key}'.")
        data = {"pos": z[pos_key]}
        if fields:
            for out_key, in_key in fields.items():
                if in_key not in z:
                    raise ValueError(f"NPZ file '{path}' does not contain key '{in_key}' for field '{out_key}'.")
                data[out_key] = z[in_key]
        else:
            data.update({k: z[k] for k in z.files if k != pos_key})
    data["size"] = np.asarray(data["pos"]).shape[0]
    return _finish(data, "read_npz")


def split_files(path):
    """``name.0, name.1, ...`` next to ``path`` (from its stem when ``path``
    exists, else from the whole name), or ``[path]`` when there are none
    (utils/func_util.py:51-80)."""
    base_dir, name = os.path.split(str(path))
    stem = name.split(".")[0] if os.path.exists(path) else name
    files = []
    while os.path.exists(os.path.join(base_dir, f"{stem}.{len(files)}")):
        files.append(os.path.join(base_dir, f"{stem}.{len(files)}"))
    if not files and os.path.exists(path):
        files = [str(path)]
    if not files:
        raise FileNotFoundError(f"Catalogue file not found: {path}")
    return files


def _record(f, dtype, count):
    """One Fortran-style record: 4-byte length, payload, 4-byte length.  The
    payload holds ``count`` values of ``dtype``; a longer record is skipped
    to its end."""
    head = np.fromfile(f, dtype=np.int32, count=1)
    if head.size != 1:
        raise EOFError("catalogue ended before a record")
    start = f.tell()
    values = np.fromfile(f, dtype=dtype, count=count)
    if values.size != count:
        raise EOFError("catalogue record shorter than expected")
    f.seek(start + int(head[0]))
    np.fromfile(f, dtype=np.int32, count=1)
    return values


_GADGET_HEADER = np.dtype([("npart", np.uint32, 6), ("massarr", np.float64, 6), ("time", np.float64),
                           ("redshift", np.float64), ("flag_sfr", np.int32), ("flag_feedback", np.int32),
                           ("npartTotal", np.int32, 6), ("flag_cooling", np.int32), ("num_files", np.int32),
                           ("BoxSize", np.float64), ("Omega0", np.float64), ("OmegaLambda", np.float64),
                           ("HubbleParam", np.float64), ("fill", np.int32, 24)])


def read_gadget(path, ptype=1, **kwargs):
    """Legacy Gadget format-1 snapshot: header, positions, velocities, IDs,
    then masses when the type's mass-table entry is zero.  Dark-matter-only
    snapshots (no gas particles), as the reference."""
    ptype = int(ptype)
    pos, vel, mass = [], [], []
    table_mass = None
    for fn in split_files(path):
        with open(fn, "rb") as f:
            h = _record(f, _GADGET_HEADER, 1)[0]
            if int(h["npart"][0]) != 0:
                raise ValueError("Only dark-matter-only legacy-format-1 Gadget snapshots are supported; "
                                 f"'{fn}' contains gas particles.")
            n = int(h["npart"][ptype])
            pos.append(_record(f, np.float32, 3 * n).reshape(-1, 3))
            vel.append(_record(f, np.float32, 3 * n).reshape(-1, 3))
            _record(f, np.uint8, 0)  # particle IDs, skipped by their record length
            from_table = float(h["massarr"][ptype]) != 0.0
            if table_mass is not None and from_table != (table_mass is not False):
                raise ValueError("Inconsistent mass table across snapshot files.")
            if from_table:
                table_mass = float(h["massarr"][ptype])
            else:
                table_mass = False
                mass.append(_record(f, np.float32, n))
    data = {"pos": np.concatenate(pos), "vel": np.concatenate(vel)}
    data["size"] = data["pos"].shape[0]
    data["mass"] = (np.full(data["size"], table_mass, dtype=np.float32) if table_mass is not False
                    else np.concatenate(mass))
    return _with_velocity_components(_finish(data, "read_gadget"))


def read_gadget_hdf5(path, ptype=1, position_scale=1.0, velocity_scale=1.0, mass_scale=1.0, load_velocity=False,
                     load_mass=False, **kwargs):
    """Gadget HDF5 snapshot(s): ``PartType{ptype}/Coordinates`` (and
    Velocities, Masses or the header MassTable), single file or split
    ``name.0.hdf5, name.1.hdf5, ...``, scaled by the given unit factors."""
    try:
        import hdf5plugin  # noqa: F401  (compressed Quijote snapshots)
    except ImportError:
        pass
    try:
        import h5py
    except ImportError as exc:
        raise ImportError("The gadget_hdf5 reader requires h5py. Compressed Quijote files may additionally "
                          "require hdf5plugin.") from exc
    p = Path(path)
    if p.is_file():
        files = [p]
    else:
        def order(fp):
            idx = fp.stem.rsplit(".", 1)[-1]
            return (0, int(idx)) if idx.isdigit() else (1, fp.name)

        files = sorted(set(p.parent.glob(f"{p.name}.*.hdf5")) | set(p.parent.glob(f"{p.name}.*.h5")), key=order)
        if not files:
            raise FileNotFoundError(f"Could not find Gadget HDF5 snapshot '{p}' or split files such as "
                                    f"'{p.name}.0.hdf5'.")
    group = f"PartType{int(ptype)}"
    pos, vel, mass = [], [], []
    for fn in files:
        with h5py.File(fn, "r") as snap:
            if group not in snap:
                continue
            g = snap[group]
            pos.append(np.asarray(g["Coordinates"][:], dtype=np.float32))
            if load_velocity:
                vel.append(np.asarray(g["Velocities"][:], dtype=np.float32))
            if load_mass:
                if "Masses" in g:
                    mass.append(np.asarray(g["Masses"][:], dtype=np.float32))
                else:
                    m = float(snap["Header"].attrs["MassTable"][int(ptype)])
                    mass.append(np.full(pos[-1].shape[0], m, dtype=np.float32))
    if not pos or sum(x.shape[0] for x in pos) == 0:
        raise ValueError(f"No particles found in HDF5 group '{group}'.")
    data = {"pos": np.concatenate(pos) * np.float32(position_scale)}
    data["size"] = data["pos"].shape[0]
    if load_velocity:
        data["vel"] = np.concatenate(vel) * np.float32(velocity_scale)
    if load_mass:
        data["mass"] = np.concatenate(mass) * np.float32(mass_scale)
    return _with_velocity_components(_finish(data, "read_gadget_hdf5"))


_GADGET_FOF_HEADER = np.dtype([("Ngroups", np.int64), ("Nsubhalos", np.int64), ("Nids", np.int64),
                               ("TotNgroups", np.int64), ("TotNsubhalos", np.int64), ("TotNids", np.int64),
                               ("num_files", np.int32), ("dummy", np.int32), ("time", np.float64),
                               ("redshift", np.float64), ("BoxSize", np.float64)])


def read_gadget_fof(path, **kwargs):
    """Legacy Gadget FoF catalogue (FoF without SUBFIND): per file a header
    record, then group lengths, masses, positions and velocities."""
    out = {}
    pos, vel, mass = [], [], []
    for fn in split_files(path):
        with open(fn, "rb") as f:
            h = _record(f, _GADGET_FOF_HEADER, 1)[0]
            if int(h["Nsubhalos"]) != 0:
                raise ValueError("The 'gadget-fof' reader supports FoF catalogues without SUBFIND only.")
            n = int(h["Ngroups"])
            _record(f, np.int32, n)
            mass.append(_record(f, np.float32, n))
            pos.append(_record(f, np.float32, 3 * n).reshape(-1, 3))
            vel.append(_record(f, np.float32, 3 * n).reshape(-1, 3))
            for k in ("TotNgroups", "TotNsubhalos", "TotNids", "num_files", "time", "redshift", "BoxSize"):
                out[k] = h[k]
    out.update({"pos": np.concatenate(pos), "vel": np.concatenate(vel), "mass": np.concatenate(mass)})
    out["size"] = out["pos"].shape[0]
    return _with_velocity_components(_finish(out, "read_gadget_fof"))


def _fof_block(f, dtype, count, swap):
    v = np.fromfile(f, dtype=dtype, count=count)
    if v.shape[0] != count:
        raise EOFError(f"FoF file ended early while reading {count} values of dtype {dtype}.")
    return v.byteswap() if swap else v


def _read_group_tab(fn, swap=False, sfr=False):
    """One group_tab file: header (Ngroups, TotNgroups, Nids: int32;
    TotNids: uint64; Nfiles: uint32), then per group length, offset, mass,
    position, velocity, two 6-vectors and optionally the SFR."""
    vec3, vec6 = np.dtype((np.float32, 3)), np.dtype((np.float32, 6))
    with open(fn, "rb") as f:
        hdr = {"Ngroups": int(_fof_block(f, np.int32, 1, swap)[0]), "TotNgroups": int(_fof_block(f, np.int32, 1, swap)[0]),
               "Nids": int(_fof_block(f, np.int32, 1, swap)[0]), "TotNids": int(_fof_block(f, np.uint64, 1, swap)[0]),
               "Nfiles": int(_fof_block(f, np.uint32, 1, swap)[0])}
        n = hdr["Ngroups"]
        part = {"len": _fof_block(f, np.int32, n, swap), "offset": _fof_block(f, np.int32, n, swap),
                "mass": _fof_block(f, np.float32, n, swap), "pos": _fof_block(f, vec3, n, swap),
                "vel": _fof_block(f, vec3, n, swap)}
        _fof_block(f, vec6, n, swap)
        _fof_block(f, vec6, n, swap)
        if sfr:
            _fof_block(f, np.float32, n, swap)
        end = f.tell()
        f.seek(0, 2)
        if end != f.tell():
            raise ValueError(f"Finished reading before EOF for FoF tab file: {fn}")
    return hdr, part


def read_fof(path, snapnum=None, redshift=0.0, fields=None, swap=False, SFR=False, prefix="/groups_", **kwargs):
    """Quijote / Pylians FoF halo catalogue: one group_tab file (its split
    siblings follow from Nfiles), or a catalogue directory with ``snapnum``
    (``<dir>/groups_NNN/group_tab_NNN.M``)."""
    src = Path(str(path))
    direct = src.is_file()
    if direct:
        first = src
    else:
        if snapnum is None:
            if not src.exists():
                raise FileNotFoundError(f"FoF input path not found: {src}")
            raise ValueError("snapnum is required when the FoF input path is a catalog directory.")
        ext = f"{int(snapnum):03d}"
        first = src / f"{str(prefix).strip('/')}{ext}" / f"group_tab_{ext}.0"
    if not first.exists():
        raise FileNotFoundError(f"FoF group_tab file not found: {first}")

    def nth(i):
        if i == 0:
            return first
        if direct:
            base, dot, idx = first.name.rpartition(".")
            if not dot or not idx.isdigit():
                raise ValueError("A direct FoF file declares multiple splits, but its filename does not end in a "
                                 f"numeric split index: {first}")
            return first.with_name(f"{base}.{i}")
        ext = f"{int(snapnum):03d}"
        return src / f"{str(prefix).strip('/')}{ext}" / f"group_tab_{ext}.{i}"

    hdr0, part0 = _read_group_tab(first, swap=bool(swap), sfr=bool(SFR))
    parts = [part0]
    for i in range(1, hdr0["Nfiles"]):
        fn = nth(i)
        if not fn.exists():
            raise FileNotFoundError(f"FoF group_tab file not found: {fn}")
        hdr, part = _read_group_tab(fn, swap=bool(swap), sfr=bool(SFR))
        if hdr["TotNgroups"] != hdr0["TotNgroups"] or hdr["Nfiles"] != hdr0["Nfiles"]:
            raise ValueError(f"Inconsistent FoF header in split file: {fn}")
        parts.append(part)
    cat = {k: np.concatenate([p[k] for p in parts], axis=0) for k in ("len", "offset", "mass", "pos", "vel")}
    if cat["pos"].shape[0] != hdr0["TotNgroups"]:
        raise ValueError(f"FoF catalog expected {hdr0['TotNgroups']} groups, but read {cat['pos'].shape[0]} groups.")
    vel = cat["vel"] * (1.0 + float(redshift))
    data = {"pos": cat["pos"] / 1e3, "vel": vel, "vel_x": vel[:, 0], "vel_y": vel[:, 1], "vel_z": vel[:, 2],
            "mass": cat["mass"] * 1e10, "npart": cat["len"], "group_offset": cat["offset"],
            "size": cat["pos"].shape[0]}
    if fields is not None:
        sel = {"pos": data["pos"], "size": data["size"]}
        for out_key, in_key in fields.items():
            if in_key not in data:
                raise ValueError(f"read_fof output does not contain field '{in_key}' for output field '{out_key}'.")
            sel[out_key] = data[in_key]
        data = sel
    return _finish(data, "read_fof")


FORMAT_READERS = {"bin": read_bin, "npz": read_npz, "gadget": read_gadget, "gadget_hdf5": read_gadget_hdf5,
                  "gadget-fof": read_gadget_fof, "fof": read_fof}


def read_particle_data(path, data_format=None, download=None, **reader_params):
    """Dispatch on the format (io/readers.py:587-611)."""
    data_format = reader_params.pop("f_format", data_format)
    data_format = reader_params.pop("format", data_format)
    if data_format == "":
        data_format = None
    if data_format is None:
        data_format = infer_format(path)
    if data_format is None:
        raise ValueError(f"Could not infer input particle format from path: {path}. Set fin.format explicitly. "
                         f"Supported formats: '{', '.join(FORMAT_READERS)}'")
    if data_format not in FORMAT_READERS:
        raise ValueError(f"Unsupported input particle format: {data_format}. Supported formats: "
                         f"'{', '.join(FORMAT_READERS)}'")
    if download is not None and not isinstance(download, dict):
        raise TypeError("download must be a mapping of resolve_data_path options.")
    from .resources import resolve_data_path

    if _is_remote(path) and not str(path).lower().startswith(("http://", "https://")):
        raise ValueError(f"Remote catalogue '{path}' needs network access; fetch it and pass the local path.")
    local = str(path)[7:] if str(path).startswith("file://") else path
    return FORMAT_READERS[data_format](resolve_data_path(local, **(download or {})), **reader_params)


def resolve_particle_value(particle_data, value_key, label="Particle value"):
    """Unit values when ``value_key`` is None, else the named 1-D field as
    float32 (io/readers.py:615-635); returns (values, key)."""
    size = int(particle_data["size"])
    if value_key is None:
        return np.ones(size, dtype=np.float32), None
    if value_key not in particle_data:
        raise KeyError(f"{label} key '{value_key}' not found in particle data. Available keys: "
                       f"{list(particle_data.keys())}.")
    v = np.asarray(particle_data[value_key])
    if v.ndim != 1 or v.shape[0] != size:
        raise ValueError(f"{label} key '{value_key}' must refer to a 1D array with length {size}, "
                         f"but got shape {v.shape}.")
    return np.ascontiguousarray(v, dtype=np.float32), value_key
