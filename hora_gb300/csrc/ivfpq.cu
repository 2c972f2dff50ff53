// ivfpq.cu — placeholder, replaced by the IVF-PQ implementation.
#include "index.h"
namespace hora {
struct IvfState {};
void ivf_state_free(IvfState *p) { delete p; }
int ivf_build(hora_index *) { return fail(HORA_ENOTIMPL, "ivfpq: not built yet"); }
int ivf_search_keys(hora_index *, int64_t, int, int64_t, const uint32_t *, SearchWorkspace &, uint64_t *, cudaStream_t) { return fail(HORA_ENOTIMPL, "ivfpq"); }
int ivf_layout(const hora_index *, uint64_t *, uint64_t *, uint64_t *, uint64_t *) { return fail(HORA_ENOTIMPL, "ivfpq"); }
int ivf_export(const hora_index *, float *, int64_t *, int64_t *, float *, uint8_t *, uint8_t *) { return fail(HORA_ENOTIMPL, "ivfpq"); }
int ivf_set_codebooks(hora_index *, const float *, const float *) { return fail(HORA_ENOTIMPL, "ivfpq"); }
int ivf_dump(const hora_index *, FILE *) { return fail(HORA_ENOTIMPL, "ivfpq"); }
int ivf_load(hora_index *, FILE *) { return fail(HORA_ENOTIMPL, "ivfpq"); }
size_t ivf_device_bytes(const hora_index *) { return 0; }
int ivf_info(const hora_index *, std::string &out) { out = "{}"; return HORA_OK; }
}
