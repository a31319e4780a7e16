// pair_products_kernel<4>: 4 spectrum pair(s) per pass (see pair_products.cuh).
#include "pair_products.cuh"

namespace hermes {

HERMES_PP_LAUNCHER(4) {
  pair_products_kernel<4><<<grid, kPPThreads, smem, s>>>(a, wins, pd, partial, k0);
  return cudaGetLastError();
}

}  // namespace hermes
