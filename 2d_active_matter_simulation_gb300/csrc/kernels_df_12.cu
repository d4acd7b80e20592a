// Double-float step and set-up kernels for transform length 4096.
#include "kernels_impl.cuh"

namespace af {
void fill_df_12(KernelTable<df> &t) { fill_range<df, 12, 12>(t); }
}  // namespace af
