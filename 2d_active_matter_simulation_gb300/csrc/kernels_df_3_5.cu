// Double-float step and set-up kernels for transform lengths 8 .. 32.
#include "kernels_impl.cuh"

namespace af {
void fill_df_3_5(KernelTable<df> &t) { fill_range<df, 3, 5>(t); }
}  // namespace af
