// Adjoint substep kernels (sm_103a) — placeholder until the adjoints land.
#include "common.cuh"

extern "C" {

int dt_substep_bwd(const dt_world* w, int f, cudaStream_t stream) {
  (void)stream;
  if (!w || f < 0 || f + 1 >= w->n_frames) return DT_ERR_ARG;
  return DT_ERR_ARG;
}

}  // extern "C"
