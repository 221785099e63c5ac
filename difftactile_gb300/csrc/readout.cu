// Action input and loss readout kernels:
//   pose control   fem_sensor.py:229-266 (set_pose_control + set_control_vel): per-vertex control
//                  velocity from the step transform dtrans_h, and its adjoint (reduction of the
//                  control-velocity adjoint to d/d(dtrans_h) plus the virtual-position adjoint)
//   marker loss    surface-node displacement field (pos - virtual pos) against a target field,
//                  the tactile readout of the press task (cf. compute_marker_motion /
//                  compute_marker_loss, grasp_plastic.py:241-256)
#include "common.cuh"

namespace {

constexpr int NT = 256;
inline int cdiv(int a, int b) { return (a + b - 1) / b; }
inline int launched() { return cudaGetLastError() == cudaSuccess ? DT_OK : DT_ERR_LAUNCH; }

__global__ void k_pose_cv(dt_world w, int s, const float* __restrict__ Ab, float inv_T, int f0, int nfr) {
  const dt_sensor& S = w.sensors[s];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.nv) return;
  const int v = S.v_off + i;
  const v3 p = f4to3(vframe(w.v_vpos, w, f0)[v]);
  v3 q;
  q.x = Ab[0] * p.x + Ab[1] * p.y + Ab[2] * p.z + Ab[3];
  q.y = Ab[4] * p.x + Ab[5] * p.y + Ab[6] * p.z + Ab[7];
  q.z = Ab[8] * p.x + Ab[9] * p.y + Ab[10] * p.z + Ab[11];
  const float4 cv = v3to4(inv_T * (q - p));
  for (int f = f0; f < f0 + nfr; ++f) vframe(w.v_cv, w, f)[v] = cv;
}

__global__ void k_pose_cv_bwd(dt_world w, int s, const float* __restrict__ Ab, float inv_T, float* Ab_bar, int f0,
                              int nfr) {
  __shared__ float red[12][NT / 32];
  const dt_sensor& S = w.sensors[s];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float g[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) g[k] = 0.f;
  if (i < S.nv) {
    const int v = S.v_off + i;
    const v3 p = f4to3(vframe(w.v_vpos, w, f0)[v]);
    v3 cb = v3{0.f, 0.f, 0.f};
    for (int f = f0; f < f0 + nfr; ++f) {  // consume: the adjoint moves into Ab_bar and vpos_bar
      float4* c = vframe(w.v_adj_cv, w, f) + v;
      cb = cb + f4to3(*c);
      *c = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    cb = inv_T * cb;
    const float pr[4] = {p.x, p.y, p.z, 1.f};
    const float cr[3] = {cb.x, cb.y, cb.z};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) g[4 * r + c] = cr[r] * pr[c];
    // cv = inv_T (A p + b - p): p_bar += (A - I)^T cb
    float4* ap = reinterpret_cast<float4*>(w.v_adj_vpos) + (size_t)(f0 & 1) * w.n_verts + v;  // frame f0's buffer
    float4 a = *ap;
    a.x += Ab[0] * cb.x + Ab[4] * cb.y + Ab[8] * cb.z - cb.x;
    a.y += Ab[1] * cb.x + Ab[5] * cb.y + Ab[9] * cb.z - cb.y;
    a.z += Ab[2] * cb.x + Ab[6] * cb.y + Ab[10] * cb.z - cb.z;
    *ap = a;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    float x = g[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    float x = 0.f;
    for (int k = 0; k < NT / 32; ++k) x += red[threadIdx.x][k];
    atomicAdd(Ab_bar + threadIdx.x, x);
  }
}

__global__ void k_marker_loss(dt_world w, int s, int f, int layer, const float4* __restrict__ target, float* loss) {
  const dt_sensor& S = w.sensors[s];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < S.nv && __ldg(w.v_layer + S.v_off + i) == layer) {
    const int v = S.v_off + i;
    const v3 d = f4to3(vframe(w.v_pos, w, f)[v]) - f4to3(vframe(w.v_vpos, w, f)[v]) - f4to3(target[i]);
    l = dot(d, d);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

__global__ void k_marker_loss_bwd(dt_world w, int s, int f, int layer, const float4* __restrict__ target, float g) {
  const dt_sensor& S = w.sensors[s];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.nv || __ldg(w.v_layer + S.v_off + i) != layer) return;
  const int v = S.v_off + i;
  const v3 d = f4to3(vframe(w.v_pos, w, f)[v]) - f4to3(vframe(w.v_vpos, w, f)[v]) - f4to3(target[i]);
  const v3 gd = (2.f * g) * d;
  const size_t V = (size_t)w.n_verts, b = (size_t)(f & 1);
  float4* ap = reinterpret_cast<float4*>(w.v_adj_pos) + b * V + v;
  float4* av = reinterpret_cast<float4*>(w.v_adj_vpos) + b * V + v;
  float4 a = *ap;
  a.x += gd.x;
  a.y += gd.y;
  a.z += gd.z;
  *ap = a;
  float4 c = *av;
  c.x -= gd.x;
  c.y -= gd.y;
  c.z -= gd.z;
  *av = c;
}

}  // namespace

extern "C" {

int dt_pose_control_vel(const dt_world* w, int s, const float* Ab, float inv_T, int f0, int nfr,
                        cudaStream_t stream) {
  if (!w || !Ab || s < 0 || s >= w->n_sensors || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames) return DT_ERR_ARG;
  k_pose_cv<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, s, Ab, inv_T, f0, nfr);
  return launched();
}

int dt_pose_control_vel_bwd(const dt_world* w, int s, const float* Ab, float inv_T, float* Ab_bar, int f0, int nfr,
                            cudaStream_t stream) {
  if (!w || !Ab || !Ab_bar || s < 0 || s >= w->n_sensors || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames)
    return DT_ERR_ARG;
  k_pose_cv_bwd<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, s, Ab, inv_T, Ab_bar, f0, nfr);
  return launched();
}

int dt_marker_loss(const dt_world* w, int s, int f, int layer, const float* target, float* loss, cudaStream_t stream) {
  if (!w || !target || !loss || s < 0 || s >= w->n_sensors || f < 0 || f >= w->n_frames) return DT_ERR_ARG;
  k_marker_loss<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, s, f, layer, reinterpret_cast<const float4*>(target),
                                                         loss);
  return launched();
}

int dt_marker_loss_bwd(const dt_world* w, int s, int f, int layer, const float* target, float loss_bar,
                       cudaStream_t stream) {
  if (!w || !target || s < 0 || s >= w->n_sensors || f < 0 || f >= w->n_frames) return DT_ERR_ARG;
  k_marker_loss_bwd<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, s, f, layer,
                                                             reinterpret_cast<const float4*>(target), loss_bar);
  return launched();
}

}  // extern "C"
