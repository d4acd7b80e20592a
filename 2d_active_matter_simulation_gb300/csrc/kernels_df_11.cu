// Double-float step and set-up kernels for transform length 2048.
#include "kernels_impl.cuh"

namespace af {
void fill_df_11(KernelTable<df> &t) { fill_range<df, 11, 11>(t); }
}  // namespace af
