// Batched relaxation kernel instantiations (device code in mm_batch_dev.cuh).
#include "mm_batch_dev.cuh"

namespace mmb {

template <typename T, int MODEL>
static void launch_relax_t(const BatchLaunch& L, int max_iter, double gtol, cudaStream_t st) {
  if (L.bt == 128) k_batch_relax<T, MODEL, 128><<<L.nctas, 128, 0, st>>>(L.a, max_iter, gtol);
  else k_batch_relax<T, MODEL, 256><<<L.nctas, 256, 0, st>>>(L.a, max_iter, gtol);
}

void launch_relax(const BatchLaunch& L, int max_iter, double gtol, cudaStream_t st) {
  if (L.prec == MM_PREC_FP32) {
    if (L.model == MM_MODEL_NANOCELL && L.simple) launch_relax_t<float, 2>(L, max_iter, gtol, st);
    else if (L.model == MM_MODEL_NANOCELL) launch_relax_t<float, 1>(L, max_iter, gtol, st);
    else launch_relax_t<float, 0>(L, max_iter, gtol, st);
  } else {
    if (L.model == MM_MODEL_NANOCELL) launch_relax_t<double, 1>(L, max_iter, gtol, st);
    else launch_relax_t<double, 0>(L, max_iter, gtol, st);
  }
}

}  // namespace mmb
