// Batched MD launch dispatch; the kernel instantiations live in mm_batch_md_*.cu.
#include "mm_batch_dev.cuh"

namespace mmb {

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
