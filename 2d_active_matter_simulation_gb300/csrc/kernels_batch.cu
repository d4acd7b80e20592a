// Batched FP32 step kernels for 128 and 256 and the assembled batch table.
#include "kernels_batch_impl.cuh"

namespace af {
void fill_batch_7_8(BatchTable &t) { FillB<7, 8>::run(t); }

const BatchTable &kernels_batch_f32()
{
    static const BatchTable t = []() {
        BatchTable b{};
        fill_batch_7_8(b);
        fill_batch_9_10(b);
        return b;
    }();
    return t;
}
}  // namespace af
