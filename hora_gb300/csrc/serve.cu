// serve.cu — placeholder for the serving loop.
#include "index.h"
extern "C" {
int hora_server_create(hora_index *const *, uint32_t, uint32_t, uint64_t, hora_server **) { return hora::fail(HORA_ENOTIMPL, "server"); }
int hora_server_free(hora_server *) { return HORA_OK; }
int hora_server_submit(hora_server *, uint32_t, const float *, uint64_t, uint64_t, uint64_t *, float *, uint64_t *) { return hora::fail(HORA_ENOTIMPL, "server"); }
int hora_server_wait(hora_server *, uint64_t, int64_t, double *) { return hora::fail(HORA_ENOTIMPL, "server"); }
int hora_server_stats(hora_server *, double *) { return hora::fail(HORA_ENOTIMPL, "server"); }
}
