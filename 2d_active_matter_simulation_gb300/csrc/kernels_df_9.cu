// Double-float step and set-up kernels for transform length 512.
#include "kernels_impl.cuh"

namespace af {
void fill_df_9(KernelTable<df> &t) { fill_range<df, 9, 9>(t); }
}  // namespace af
