// Batched FP32 step kernels for 512 and 1024.
#include "kernels_batch_impl.cuh"

namespace af {
void fill_batch_9_10(BatchTable &t) { FillB<9, 10>::run(t); }
}  // namespace af
