// Batched MD kernel instantiation: FP32 cells, nanocell model.
#include "mm_batch_dev.cuh"

namespace mmb {

template <>
void launch_md_t<float, 1>(const BatchLaunch& L, const BMD& p, cudaStream_t st) {
  if (L.bt == 128) k_batch_md<float, 1, 128><<<L.nctas, 128, 0, st>>>(L.a, p);
  else k_batch_md<float, 1, 256><<<L.nctas, 256, 0, st>>>(L.a, p);
}

}  // namespace mmb
