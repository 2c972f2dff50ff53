// nprobe_mlp.cu — placeholder for the learned-nprobe model.
#include "index.h"
namespace hora {
struct NprobeModel {};
void nprobe_model_free(NprobeModel *p) { delete p; }
}
extern "C" {
int hora_ivfpq_train_nprobe(hora_index *, const float *, uint64_t, uint64_t, double, uint64_t, double *) { return hora::fail(HORA_ENOTIMPL, "learned nprobe"); }
int hora_ivfpq_nprobe_features(hora_index *, const float *, uint64_t, float *) { return hora::fail(HORA_ENOTIMPL, "learned nprobe"); }
int hora_ivfpq_predict_nprobe(hora_index *, const float *, uint64_t, uint32_t *) { return hora::fail(HORA_ENOTIMPL, "learned nprobe"); }
int hora_mlp_forward(const float *, uint64_t, uint64_t, uint64_t, const float *, uint64_t, float *) { return hora::fail(HORA_ENOTIMPL, "mlp"); }
int hora_mlp_loss_grad(const float *, uint64_t, uint64_t, uint64_t, const float *, const float *, uint64_t, float, float *, float *) { return hora::fail(HORA_ENOTIMPL, "mlp"); }
}
