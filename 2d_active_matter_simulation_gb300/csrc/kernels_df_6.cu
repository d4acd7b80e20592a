// Double-float step and set-up kernels for transform length 64.
#include "kernels_impl.cuh"

namespace af {
void fill_df_6(KernelTable<df> &t) { fill_range<df, 6, 6>(t); }
}  // namespace af
