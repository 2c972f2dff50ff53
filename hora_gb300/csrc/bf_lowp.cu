// bf_lowp.cu — placeholder for the low-precision scoring path.
#include "index.h"
namespace hora {
struct LowpState {};
void lowp_state_free(LowpState *p) { delete p; }
int lowp_search_keys(hora_index *, int64_t, int, SearchWorkspace &, uint64_t *, cudaStream_t) { return fail(HORA_ENOTIMPL, "low precision: not built yet"); }
}
