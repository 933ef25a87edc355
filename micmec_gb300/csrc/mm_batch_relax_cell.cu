// Batched relaxation with cell DOFs: kernel instantiations (device code in mm_batch_dev.cuh).
#include "mm_batch_dev.cuh"

namespace mmb {

template <typename T, int MODEL>
static void launch_t(const BatchLaunch& L, const CellRelax& r, cudaStream_t st) {
  if (L.bt == 128) k_batch_relax_cell<T, MODEL, 128><<<L.nctas, 128, 0, st>>>(L.a, r);
  else k_batch_relax_cell<T, MODEL, 256><<<L.nctas, 256, 0, st>>>(L.a, r);
}

void launch_relax_cell(const BatchLaunch& L, const CellRelax& r, cudaStream_t st) {
  if (L.prec == MM_PREC_FP32) {
    if (L.model == MM_MODEL_NANOCELL && L.simple) launch_t<float, 2>(L, r, st);
    else if (L.model == MM_MODEL_NANOCELL) launch_t<float, 1>(L, r, st);
    else launch_t<float, 0>(L, r, st);
  } else {
    if (L.model == MM_MODEL_NANOCELL) launch_t<double, 1>(L, r, st);
    else launch_t<double, 0>(L, r, st);
  }
}

}  // namespace mmb
