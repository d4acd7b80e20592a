// Double-float step and set-up kernels for transform length 256.
#include "kernels_impl.cuh"

namespace af {
void fill_df_8(KernelTable<df> &t) { fill_range<df, 8, 8>(t); }
}  // namespace af
