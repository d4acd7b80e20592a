// Double-float step and set-up kernels for transform length 1024.
#include "kernels_impl.cuh"

namespace af {
void fill_df_10(KernelTable<df> &t) { fill_range<df, 10, 10>(t); }
}  // namespace af
