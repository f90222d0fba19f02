// Search kernels: CRS, fast form.
#define SEMB_WIDE_WINDOWS 0
#include "search_inst.cuh"

namespace semb {
SearchEntry search_entry_crs_fast(int w, int variant) { return search_entry<METHOD_CRS, FORM_FAST>(w, variant); }
}  // namespace semb
