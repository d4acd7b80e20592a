// Work-list forms of the FP32 step kernels for ragged batches: one launch per
// pass covers the runs of every size class.  Each CTA reads its work item --
// (run, CTA index within that run's own launch, log2 of the transform
// length) -- and runs the kernel body of that length: the row pass with
// radix-8 passes (RowPass) and the narrow column pass (ColPass, VAR 1), whose
// CTAs have 128 threads at every length from 128 to 1024, so one block size
// serves the whole list.  The host sorts the list by grid size, largest
// first, so the block scheduler hands out the longest items first.
#include "kernels_impl.cuh"

namespace af {

namespace {

template <int LOG, int MODE>
constexpr size_t col_smem() { return ColPass<float, LOG, MODE, 1>::smem_bytes(); }
template <int LOG>
constexpr size_t row_smem() { return RowPass<float, LOG>::smem_bytes(); }
constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }

constexpr size_t QROW_SMEM = cmax(cmax(row_smem<7>(), row_smem<8>()), cmax(row_smem<9>(), row_smem<10>()));
constexpr size_t QCOL_SMEM =
    cmax(cmax(col_smem<7, 1>(), col_smem<8, 1>()), cmax(col_smem<9, 1>(), col_smem<10, 1>()));

static_assert(RowPass<float, 7>::THREADS == 128 && RowPass<float, 10>::THREADS == 128, "row CTAs of 128");
static_assert(ColPass<float, 7, 1, 1>::THREADS == 128 && ColPass<float, 10, 1, 1>::THREADS == 128,
              "column CTAs of 128");

__global__ void __launch_bounds__(128, 4) k_row_q(const StepArgs<float> *__restrict__ args, const WorkItem *items)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const WorkItem it = items[blockIdx.x];
    const StepArgs<float> a = args[it.arg];
    auto sync = []() { __syncthreads(); };
    switch (it.log) {
    case 7: RowPass<float, 7>::body(a, threadIdx.x, it.block, smem, sync); break;
    case 8: RowPass<float, 8>::body(a, threadIdx.x, it.block, smem, sync); break;
    case 9: RowPass<float, 9>::body(a, threadIdx.x, it.block, smem, sync); break;
    default: RowPass<float, 10>::body(a, threadIdx.x, it.block, smem, sync); break;
    }
}

template <int MODE>
__global__ void __launch_bounds__(128, 4) k_col_q(const StepArgs<float> *__restrict__ args, const WorkItem *items)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const WorkItem it = items[blockIdx.x];
    const StepArgs<float> a = args[it.arg];
    auto sync = []() { __syncthreads(); };
    switch (it.log) {
    case 7: ColPass<float, 7, MODE, 1>::body(a, threadIdx.x, it.block, smem, sync); break;
    case 8: ColPass<float, 8, MODE, 1>::body(a, threadIdx.x, it.block, smem, sync); break;
    case 9: ColPass<float, 9, MODE, 1>::body(a, threadIdx.x, it.block, smem, sync); break;
    default: ColPass<float, 10, MODE, 1>::body(a, threadIdx.x, it.block, smem, sync); break;
    }
}

}  // namespace

const QueueTable &kernels_queue_f32()
{
    static const QueueTable t = []() {
        QueueTable q{};
        q.row = k_row_q;
        q.col[1] = k_col_q<1>;
        q.col[2] = k_col_q<2>;
        q.col[3] = k_col_q<3>;
        q.col[4] = k_col_q<4>;
        q.row_smem = QROW_SMEM;
        q.col_smem = QCOL_SMEM;
        return q;
    }();
    return t;
}

}  // namespace af
