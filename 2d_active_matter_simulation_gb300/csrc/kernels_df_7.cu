// Double-float step and set-up kernels for transform length 128.
#include "kernels_impl.cuh"

namespace af {
void fill_df_7(KernelTable<df> &t) { fill_range<df, 7, 7>(t); }
}  // namespace af
