// Search kernels: CMP, fast form.
#define SEMB_WIDE_WINDOWS 1
#include "search_inst.cuh"

namespace semb {
SearchEntry search_entry_cmp_fast(int w, int variant) { return search_entry<METHOD_CMP, FORM_FAST>(w, variant); }
}  // namespace semb
