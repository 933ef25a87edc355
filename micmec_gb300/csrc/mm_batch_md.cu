// Batched MD kernel instantiations (device code in mm_batch_dev.cuh).
#include "mm_batch_dev.cuh"

namespace mmb {

template <typename T, int MODEL>
static void launch_md_t(const BatchLaunch& L, const BMD& p, cudaStream_t st) {
  if (L.bt == 128) k_batch_md<T, MODEL, 128><<<L.nctas, 128, 0, st>>>(L.a, p);
  else k_batch_md<T, MODEL, 256><<<L.nctas, 256, 0, st>>>(L.a, p);
}

void launch_md(const BatchLaunch& L, const BMD& p, cudaStream_t st) {
  if (L.prec == MM_PREC_FP32) {
    if (L.model == MM_MODEL_NANOCELL && L.simple) launch_md_t<float, 2>(L, p, st);
    else if (L.model == MM_MODEL_NANOCELL) launch_md_t<float, 1>(L, p, st);
    else launch_md_t<float, 0>(L, p, st);
  } else {
    if (L.model == MM_MODEL_NANOCELL) launch_md_t<double, 1>(L, p, st);
    else launch_md_t<double, 0>(L, p, st);
  }
}

}  // namespace mmb
