// Action input and loss readout kernels:
//   pose control   fem_sensor.py:229-266 (set_pose_control + set_control_vel): per-vertex control
//                  velocity from the step transform dtrans_h, and its adjoint (reduction of the
//                  control-velocity adjoint to d/d(dtrans_h) plus the virtual-position adjoint)
//   marker loss    surface-node displacement field (pos - virtual pos) against a target field,
//                  the tactile readout of the press task (cf. compute_marker_motion /
//                  compute_marker_loss, grasp_plastic.py:241-256)
//   contact force  compute_contact_force, grasp_plastic.py:218-229: sum over the surface triangles of
//                  1/6 of the contact force on each of its three vertices
//   rigid match    compute_COM + compute_H, multi_obj.py:309-326: centres of the rigid particles at
//                  frames f and f+1 (sums divided by the env's particle count, as the reference) and
//                  H = sum (x_f - c0)(x_{f+1} - c1)^T over them; adjoint scattered back to both frames
//   markers        extract_markers, fem_sensor.py:161-187: surface nodes (current and virtual) into the
//                  sensor frame (inv_trans_h), fisheye projection project_3d_2d
//                  (sensor_model/fisheye_model.py:12-30), k-nearest inverse-distance interpolation to
//                  the marker set
#include "common.cuh"

namespace {

constexpr int NT = 256;
inline int cdiv(int a, int b) { return (a + b - 1) / b; }
inline int launched() { return launch_status(cudaGetLastError()); }

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

// every sensor at once: Ab [n_sensors][12], one row per sensor
__global__ void k_pose_cv_all(dt_world w, const float* __restrict__ Ab, float inv_T, int f0, int nfr) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= w.n_verts) return;
  const float* A = Ab + 12 * __ldg(w.v_sensor + v);
  const v3 p = f4to3(vframe(w.v_vpos, w, f0)[v]);
  v3 q;
  q.x = A[0] * p.x + A[1] * p.y + A[2] * p.z + A[3];
  q.y = A[4] * p.x + A[5] * p.y + A[6] * p.z + A[7];
  q.z = A[8] * p.x + A[9] * p.y + A[10] * p.z + A[11];
  const float4 cv = v3to4(inv_T * (q - p));
  for (int f = f0; f < f0 + nfr; ++f) vframe(w.v_cv, w, f)[v] = cv;
}

// one thread per (frame, vertex): everything below is linear in the per-frame adjoint cvb_f, so the
// frames are summed by the reductions (Ab_bar) and atomics (v_adj_vpos) instead of a loop per vertex
__global__ void k_pose_cv_bwd(dt_world w, int s, const float* __restrict__ Ab, float inv_T, float* Ab_bar, int f0,
                              int nfr) {
  __shared__ float red[12][NT / 32];
  const dt_sensor& S = w.sensors[s];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = f0 + blockIdx.y;
  float g[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) g[k] = 0.f;
  if (i < S.nv) {
    const int v = S.v_off + i;
    const v3 p = f4to3(vframe(w.v_vpos, w, f0)[v]);
    float4* c = vframe(w.v_adj_cv, w, f) + v;  // consumed: the adjoint moves into Ab_bar and vpos_bar
    const v3 cb = inv_T * f4to3(*c);
    *c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (cb.x != 0.f || cb.y != 0.f || cb.z != 0.f) {
      const float pr[4] = {p.x, p.y, p.z, 1.f};
      const float cr[3] = {cb.x, cb.y, cb.z};
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) g[4 * r + cc] = cr[r] * pr[cc];
      // cv = inv_T (A p + b - p): p_bar += (A - I)^T cb, into frame f0's buffer
      float4* ap = reinterpret_cast<float4*>(w.v_adj_vpos) + (size_t)(f0 & 1) * w.n_verts + v;
      red_add_v4(ap, make_float4(Ab[0] * cb.x + Ab[4] * cb.y + Ab[8] * cb.z - cb.x,
                                 Ab[1] * cb.x + Ab[5] * cb.y + Ab[9] * cb.z - cb.y,
                                 Ab[2] * cb.x + Ab[6] * cb.y + Ab[10] * cb.z - cb.z, 0.f));
    }
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
    if (x != 0.f) atomicAdd(Ab_bar + threadIdx.x, x);
  }
}

// every sensor at once (Ab, Ab_bar [n_sensors][12]): one thread per (frame, vertex) over all
// vertices; vertices are sensor-contiguous, so a warp whose vertices share one sensor sums its 12
// partial products with shuffles before its atomics, and a CTA that lies in one sensor sums its warps
// in shared memory first
__global__ void k_pose_cv_bwd_all(dt_world w, const float* __restrict__ Ab, float inv_T, float* Ab_bar, int f0,
                                  int nfr) {
  __shared__ float red[12][NT / 32];
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = f0 + blockIdx.y;
  float g[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) g[k] = 0.f;
  int s = -1;
  if (v < w.n_verts) {
    s = __ldg(w.v_sensor + v);
    const float* A = Ab + 12 * s;
    const v3 p = f4to3(vframe(w.v_vpos, w, f0)[v]);
    float4* c = vframe(w.v_adj_cv, w, f) + v;  // consumed: the adjoint moves into Ab_bar and vpos_bar
    const v3 cb = inv_T * f4to3(*c);
    *c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (cb.x != 0.f || cb.y != 0.f || cb.z != 0.f) {
      const float pr[4] = {p.x, p.y, p.z, 1.f};
      const float cr[3] = {cb.x, cb.y, cb.z};
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) g[4 * r + cc] = cr[r] * pr[cc];
      float4* ap = reinterpret_cast<float4*>(w.v_adj_vpos) + (size_t)(f0 & 1) * w.n_verts + v;
      red_add_v4(ap, make_float4(A[0] * cb.x + A[4] * cb.y + A[8] * cb.z - cb.x,
                                 A[1] * cb.x + A[5] * cb.y + A[9] * cb.z - cb.y,
                                 A[2] * cb.x + A[6] * cb.y + A[10] * cb.z - cb.z, 0.f));
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // the CTA's vertices [v_first, v_last] lie in one sensor iff the two ends do (contiguous sensors)
  const int v_first = blockIdx.x * blockDim.x;
  const int v_last = min(v_first + (int)blockDim.x, w.n_verts) - 1;
  const int s_cta = __ldg(w.v_sensor + v_first);
  const bool cta_one = s_cta == __ldg(w.v_sensor + v_last);
  const int s0 = __shfl_sync(0xffffffffu, s, 0);
  const bool warp_one = __all_sync(0xffffffffu, s == s0 || s < 0);
  if (warp_one) {
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      float x = g[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      g[k] = x;
    }
  }
  if (cta_one) {  // block-uniform
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < 12; ++k) red[k][wid] = g[k];  // every warp of the CTA is single-sensor here
    }
    __syncthreads();
    if (threadIdx.x < 12) {
      float x = 0.f;
      for (int k = 0; k < NT / 32; ++k) x += red[threadIdx.x][k];
      if (x != 0.f) atomicAdd(Ab_bar + 12 * s_cta + threadIdx.x, x);
    }
  } else if (warp_one) {
    if (lane == 0 && s0 >= 0) {
#pragma unroll
      for (int k = 0; k < 12; ++k)
        if (g[k] != 0.f) atomicAdd(Ab_bar + 12 * s0 + k, g[k]);
    }
  } else if (s >= 0) {
#pragma unroll
    for (int k = 0; k < 12; ++k)
      if (g[k] != 0.f) atomicAdd(Ab_bar + 12 * s + k, g[k]);
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

// ---------------------------------------------------------------- affine control velocity
// gripper fingers (fem_sensor1/2_set_control_vel, gripper_kinematics.py:196-216): per frame
// f0 + k, cv = D_k[:, 0:3] src + D_k[:, 3] with D_k = rows 0..2 of (F_{f+1} - F_f) T0^-1 / dt
__global__ void k_affine_cv(dt_world w, int s, const float* __restrict__ D, const float4* __restrict__ src, int f0,
                            int nfr) {
  const dt_sensor& S = w.sensors[s];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.nv) return;
  const int v = S.v_off + i;
  const v3 p = f4to3(src[v]);
  for (int k = 0; k < nfr; ++k) {
    const float* A = D + 12 * k;
    const v3 c = v3{A[0] * p.x + A[1] * p.y + A[2] * p.z + A[3], A[4] * p.x + A[5] * p.y + A[6] * p.z + A[7],
                    A[8] * p.x + A[9] * p.y + A[10] * p.z + A[11]};
    vframe(w.v_cv, w, f0 + k)[v] = v3to4(c);
  }
}

// D_b[k] += sum_i cvb_i(f0 + k) [src_i, 1]^T; the control-velocity adjoint is consumed
__global__ void k_affine_cv_bwd(dt_world w, int s, const float4* __restrict__ src, int f0, int nfr, float* Db) {
  __shared__ float red[12][NT / 32];
  const dt_sensor& S = w.sensors[s];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v3 p = v3{0.f, 0.f, 0.f};
  if (i < S.nv) p = f4to3(src[S.v_off + i]);
  for (int k = 0; k < nfr; ++k) {
    v3 cb = v3{0.f, 0.f, 0.f};
    if (i < S.nv) {
      float4* c = vframe(w.v_adj_cv, w, f0 + k) + S.v_off + i;
      cb = f4to3(*c);
      *c = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float pr[4] = {p.x, p.y, p.z, 1.f};
    const float cr[3] = {cb.x, cb.y, cb.z};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float x = cr[r] * pr[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[4 * r + c][wid] = x;
      }
    __syncthreads();
    if (threadIdx.x < 12) {
      float x = 0.f;
      for (int q = 0; q < NT / 32; ++q) x += red[threadIdx.x][q];
      atomicAdd(Db + 12 * k + threadIdx.x, x);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- rigid shape matching
// out[0..2] += sum x_f / N, out[4..6] += sum x_{f+1} / N over env e's particles of material `mat`
__global__ void k_rigid_com(dt_world w, int e, int mat, int f, float* out) {
  __shared__ float red[6][NT / 32];
  const dt_env& E = w.envs[e];
  const int p = E.p_begin + blockIdx.x * blockDim.x + threadIdx.x;
  const float invN = 1.f / (float)(E.p_end - E.p_begin);
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (p < E.p_end && __ldg(w.p_mat + p) == mat) {
    const float4 a = __ldg(pplane(w, f, 0) + p), b = __ldg(pplane(w, f + 1, 0) + p);
    v[0] = a.x * invN;
    v[1] = a.y * invN;
    v[2] = a.z * invN;
    v[3] = b.x * invN;
    v[4] = b.y * invN;
    v[5] = b.z * invN;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane == 0) red[k][wid] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    float x = 0.f;
    for (int q = 0; q < NT / 32; ++q) x += red[threadIdx.x][q];
    atomicAdd(out + (threadIdx.x < 3 ? threadIdx.x : threadIdx.x + 1), x);
  }
}

// out[8..16] += sum (x_f - c0)(x_{f+1} - c1)^T (row-major), c0 = com[0..2], c1 = com[4..6]
__global__ void k_rigid_H(dt_world w, int e, int mat, int f, const float* __restrict__ com, float* out) {
  __shared__ float red[9][NT / 32];
  const dt_env& E = w.envs[e];
  const int p = E.p_begin + blockIdx.x * blockDim.x + threadIdx.x;
  float h[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) h[k] = 0.f;
  if (p < E.p_end && __ldg(w.p_mat + p) == mat) {
    const float4 a4 = __ldg(pplane(w, f, 0) + p), b4 = __ldg(pplane(w, f + 1, 0) + p);
    const float a[3] = {a4.x - com[0], a4.y - com[1], a4.z - com[2]};
    const float b[3] = {b4.x - com[4], b4.y - com[5], b4.z - com[6]};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) h[3 * r + c] = a[r] * b[c];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h[k] += __shfl_xor_sync(0xffffffffu, h[k], o);
    if (lane == 0) red[k][wid] = h[k];
  }
  __syncthreads();
  if (threadIdx.x < 9) {
    float x = 0.f;
    for (int q = 0; q < NT / 32; ++q) x += red[threadIdx.x][q];
    atomicAdd(out + 8 + threadIdx.x, x);
  }
}

// adjoint of H for the rigid particles: frame f (part 0): x_bar += Hb (b - bbar); frame f+1
// (part 1): x_bar += Hb^T (a - abar); abar / bbar = sums of a / b divided by N (aux[0..2] / [4..6])
__global__ void k_rigid_H_bwd(dt_world w, int e, int mat, int f, int part, const float* __restrict__ com,
                              const float* __restrict__ aux, const float* __restrict__ Hb) {
  const dt_env& E = w.envs[e];
  const int p = E.p_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= E.p_end || __ldg(w.p_mat + p) != mat) return;
  const int g = part == 0 ? f : f + 1;
  const float4 a4 = __ldg(pplane(w, f, 0) + p), b4 = __ldg(pplane(w, f + 1, 0) + p);
  v3 d;
  if (part == 0) {
    const float b[3] = {b4.x - com[4] - aux[4], b4.y - com[5] - aux[5], b4.z - com[6] - aux[6]};
    d = v3{Hb[0] * b[0] + Hb[1] * b[1] + Hb[2] * b[2], Hb[3] * b[0] + Hb[4] * b[1] + Hb[5] * b[2],
           Hb[6] * b[0] + Hb[7] * b[1] + Hb[8] * b[2]};
  } else {
    const float a[3] = {a4.x - com[0] - aux[0], a4.y - com[1] - aux[1], a4.z - com[2] - aux[2]};
    d = v3{Hb[0] * a[0] + Hb[3] * a[1] + Hb[6] * a[2], Hb[1] * a[0] + Hb[4] * a[1] + Hb[7] * a[2],
           Hb[2] * a[0] + Hb[5] * a[1] + Hb[8] * a[2]};
  }
  float4* ax = reinterpret_cast<float4*>(w.p_adj) + (size_t)(g & 1) * 6 * w.n_particles + p;
  const float4 x = *ax;
  *ax = make_float4(x.x + d.x, x.y + d.y, x.z + d.z, x.w);
}

// aux[0..2] = sum (x_f - c0) / N, aux[4..6] = sum (x_{f+1} - c1) / N over the rigid particles
__global__ void k_rigid_centred_means(dt_world w, int e, int mat, int f, const float* __restrict__ com, float* aux) {
  __shared__ float red[6][NT / 32];
  const dt_env& E = w.envs[e];
  const int p = E.p_begin + blockIdx.x * blockDim.x + threadIdx.x;
  const float invN = 1.f / (float)(E.p_end - E.p_begin);
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (p < E.p_end && __ldg(w.p_mat + p) == mat) {
    const float4 a = __ldg(pplane(w, f, 0) + p), b = __ldg(pplane(w, f + 1, 0) + p);
    v[0] = (a.x - com[0]) * invN;
    v[1] = (a.y - com[1]) * invN;
    v[2] = (a.z - com[2]) * invN;
    v[3] = (b.x - com[4]) * invN;
    v[4] = (b.y - com[5]) * invN;
    v[5] = (b.z - com[6]) * invN;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane == 0) red[k][wid] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    float x = 0.f;
    for (int q = 0; q < NT / 32; ++q) x += red[threadIdx.x][q];
    atomicAdd(aux + (threadIdx.x < 3 ? threadIdx.x : threadIdx.x + 1), x);
  }
}

// ---------------------------------------------------------------- contact force readout
__global__ void k_contact_force(dt_world w, int s, int f, float* out) {
  __shared__ float red[3][NT / 32];
  const dt_sensor& S = w.sensors[s];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  v3 a = v3{0.f, 0.f, 0.f};
  if (t < S.nf) {
    const int4 tr = __ldg(reinterpret_cast<const int4*>(w.tris) + S.f_off + t);
    const float4* E = vframe(w.v_ext, w, f);
    const float k = 1.f / 6.f;
    a = (k * f4to3(E[tr.x]) + k * f4to3(E[tr.y])) + k * f4to3(E[tr.z]);
  }
  float c[3] = {a.x, a.y, a.z};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c[k] += __shfl_xor_sync(0xffffffffu, c[k], o);
    if (lane == 0) red[k][wid] = c[k];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    float x = 0.f;
    for (int k = 0; k < NT / 32; ++k) x += red[threadIdx.x][k];
    atomicAdd(out + threadIdx.x, x);
  }
}

__global__ void k_contact_force_bwd(dt_world w, int s, const float* __restrict__ gb) {
  const dt_sensor& S = w.sensors[s];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.nf) return;
  const int4 tr = __ldg(reinterpret_cast<const int4*>(w.tris) + S.f_off + t);
  const float k = 1.f / 6.f;
  const float4 g = make_float4(k * gb[0], k * gb[1], k * gb[2], 0.f);
  float4* ae = reinterpret_cast<float4*>(w.v_adj_ext);
  red_add_v4(ae + tr.x, g);
  red_add_v4(ae + tr.y, g);
  red_add_v4(ae + tr.z, g);
}

// ---------------------------------------------------------------- markers
struct Proj {
  float2 p;
  // intermediates for the adjoint
  v3 a;
  float an, c, craw, om, r;
};

// project_3d_2d (fisheye_model.py:12-30): equidistant fisheye r = m f theta around the optical axis z
DT_DEV Proj fisheye(v3 a, const dt_fisheye& cam) {
  Proj o;
  a.z += cam.plane;
  o.a = a;
  o.an = sqrtf(dot(a, a) + 1e-10f);
  o.craw = a.z / o.an;
  o.c = fmaxf(-1.f, fminf(1.f, o.craw));
  const float th = acosf(o.c);
  o.om = atan2f(a.y, a.x + 1e-8f) + 3.14159265358979f;
  o.r = cam.m * cam.f * th;
  o.p = make_float2(o.r * cosf(o.om) + cam.cx, o.r * sinf(o.om) + cam.cy);
  return o;
}

// adjoint of fisheye: d/da (the plane shift has unit derivative)
DT_DEV v3 fisheye_bwd(const Proj& o, const dt_fisheye& cam, float2 pb) {
  const float co = cosf(o.om), so = sinf(o.om);
  const float rb = pb.x * co + pb.y * so;
  const float omb = -pb.x * o.r * so + pb.y * o.r * co;
  const float thb = cam.m * cam.f * rb;
  // acos'(c) = -1 / sqrt(1 - c^2); no derivative where the cosine was clamped
  const float cb = (o.craw > -1.f && o.craw < 1.f) ? -thb / sqrtf(fmaxf(1.f - o.c * o.c, 1e-30f)) : 0.f;
  const float X = o.a.x + 1e-8f, Y = o.a.y;
  const float den = X * X + Y * Y;
  v3 ab = v3{den > 0.f ? -omb * Y / den : 0.f, den > 0.f ? omb * X / den : 0.f, 0.f};
  // c = a.z / an, an = sqrt(|a|^2 + 1e-10)
  ab.z += cb / o.an;
  const float anb = -cb * o.a.z / (o.an * o.an);
  ab = ab + (anb / o.an) * o.a;
  return ab;
}

// sensor-frame camera coordinates of world point x: inv_trans_h rows 0..2 applied to (x, 1), then
// (x, z, y) (fem_sensor.py:168-172)
DT_DEV v3 cam_coords(const float* M, v3 x) {
  const float ix = M[0] * x.x + M[1] * x.y + M[2] * x.z + M[3];
  const float iy = M[4] * x.x + M[5] * x.y + M[6] * x.z + M[7];
  const float iz = M[8] * x.x + M[9] * x.y + M[10] * x.z + M[11];
  return v3{ix, iz, iy};
}

__global__ void k_markers(dt_world w, int s, int f, const int* __restrict__ surf, const int* __restrict__ idx,
                          const float* __restrict__ wts, int K, int M, const float* __restrict__ Mi, dt_fisheye cam,
                          float2* pred, float2* virt) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const dt_sensor& S = w.sensors[s];
  const float4* P = vframe(w.v_pos, w, f);
  const float4* VP = vframe(w.v_vpos, w, f);
  float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
  for (int k = 0; k < K; ++k) {
    const int v = S.v_off + __ldg(surf + __ldg(idx + m * K + k));
    const float wk = __ldg(wts + m * K + k);
    const Proj pp = fisheye(cam_coords(Mi, f4to3(P[v])), cam);
    const Proj pv = fisheye(cam_coords(Mi, f4to3(VP[v])), cam);
    a.x += wk * pp.p.x;
    a.y += wk * pp.p.y;
    b.x += wk * pv.p.x;
    b.y += wk * pv.p.y;
  }
  pred[m] = a;
  virt[m] = b;
}

__global__ void k_markers_bwd(dt_world w, int s, int f, const int* __restrict__ surf, const int* __restrict__ idx,
                              const float* __restrict__ wts, int K, int M, const float* __restrict__ Mi,
                              dt_fisheye cam, const float2* __restrict__ pred_b, const float2* __restrict__ virt_b,
                              float* Mi_b) {
  __shared__ float red[12][NT / 32];
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  float g[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) g[k] = 0.f;
  if (m < M) {
    const dt_sensor& S = w.sensors[s];
    const size_t V = (size_t)w.n_verts, cb = (size_t)(f & 1);
    const float4* P = vframe(w.v_pos, w, f);
    const float4* VP = vframe(w.v_vpos, w, f);
    float4* aP = reinterpret_cast<float4*>(w.v_adj_pos) + cb * V;
    float4* aVP = reinterpret_cast<float4*>(w.v_adj_vpos) + cb * V;
    const float2 gp = pred_b ? pred_b[m] : make_float2(0.f, 0.f);
    const float2 gv = virt_b ? virt_b[m] : make_float2(0.f, 0.f);
    for (int k = 0; k < K; ++k) {
      const int v = S.v_off + __ldg(surf + __ldg(idx + m * K + k));
      const float wk = __ldg(wts + m * K + k);
      for (int which = 0; which < 2; ++which) {
        const float2 lb = which == 0 ? gp : gv;
        if (lb.x == 0.f && lb.y == 0.f) continue;
        const v3 x = f4to3(which == 0 ? P[v] : VP[v]);
        const Proj pr = fisheye(cam_coords(Mi, x), cam);
        const v3 ab = fisheye_bwd(pr, cam, make_float2(wk * lb.x, wk * lb.y));
        // cam = (ix, iz, iy)
        const float ib[3] = {ab.x, ab.z, ab.y};
        const float hx[4] = {x.x, x.y, x.z, 1.f};
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) g[4 * r + c] += ib[r] * hx[c];
        const v3 xb = v3{Mi[0] * ib[0] + Mi[4] * ib[1] + Mi[8] * ib[2], Mi[1] * ib[0] + Mi[5] * ib[1] + Mi[9] * ib[2],
                         Mi[2] * ib[0] + Mi[6] * ib[1] + Mi[10] * ib[2]};
        red_add_v4((which == 0 ? aP : aVP) + v, v3to4(xb));
      }
    }
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
  if (threadIdx.x < 12 && Mi_b) {
    float x = 0.f;
    for (int k = 0; k < NT / 32; ++k) x += red[threadIdx.x][k];
    atomicAdd(Mi_b + threadIdx.x, x);
  }
}

}  // namespace

extern "C" {

int dt_affine_control_vel(const dt_world* w, int s, const float* D, const float* src, int f0, int nfr,
                          cudaStream_t stream) {
  if (!w || !D || !src || s < 0 || s >= w->n_sensors || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames) return DT_ERR_ARG;
  k_affine_cv<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, s, D, reinterpret_cast<const float4*>(src), f0, nfr);
  return launched();
}

int dt_affine_control_vel_bwd(const dt_world* w, int s, const float* src, int f0, int nfr, float* D_b,
                              cudaStream_t stream) {
  if (!w || !D_b || !src || s < 0 || s >= w->n_sensors || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames)
    return DT_ERR_ARG;
  k_affine_cv_bwd<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, s, reinterpret_cast<const float4*>(src), f0, nfr,
                                                           D_b);
  return launched();
}

int dt_rigid_match(const dt_world* w, int e, int mat, int f, float* out, cudaStream_t stream) {
  if (!w || !out || e < 0 || e >= w->n_envs || f < 0 || f + 1 >= w->n_frames) return DT_ERR_ARG;
  if (note_error(cudaMemsetAsync(out, 0, 20 * sizeof(float), stream)) != cudaSuccess) return DT_ERR_LAUNCH;
  const int nb = cdiv(w->n_particles > 0 ? w->n_particles : 1, NT);
  k_rigid_com<<<nb, NT, 0, stream>>>(*w, e, mat, f, out);
  k_rigid_H<<<nb, NT, 0, stream>>>(*w, e, mat, f, out, out);
  return launched();
}

int dt_rigid_match_bwd(const dt_world* w, int e, int mat, int f, int part, const float* out, const float* H_b,
                       float* scratch, cudaStream_t stream) {
  if (!w || !out || !H_b || !scratch || e < 0 || e >= w->n_envs || f < 0 || f + 1 >= w->n_frames || part < 0 ||
      part > 1)
    return DT_ERR_ARG;
  if (note_error(cudaMemsetAsync(scratch, 0, 8 * sizeof(float), stream)) != cudaSuccess) return DT_ERR_LAUNCH;
  const int nb = cdiv(w->n_particles > 0 ? w->n_particles : 1, NT);
  k_rigid_centred_means<<<nb, NT, 0, stream>>>(*w, e, mat, f, out, scratch);
  k_rigid_H_bwd<<<nb, NT, 0, stream>>>(*w, e, mat, f, part, out, scratch, H_b);
  return launched();
}

int dt_contact_force(const dt_world* w, int s, int f, float* out, cudaStream_t stream) {
  if (!w || !out || s < 0 || s >= w->n_sensors || f < 0 || f >= w->n_frames) return DT_ERR_ARG;
  k_contact_force<<<cdiv(w->max_sensor_tris > 0 ? w->max_sensor_tris : 1, NT), NT, 0, stream>>>(*w, s, f, out);
  return launched();
}

int dt_contact_force_bwd(const dt_world* w, int s, const float* out_b, cudaStream_t stream) {
  if (!w || !out_b || s < 0 || s >= w->n_sensors) return DT_ERR_ARG;
  k_contact_force_bwd<<<cdiv(w->max_sensor_tris > 0 ? w->max_sensor_tris : 1, NT), NT, 0, stream>>>(*w, s, out_b);
  return launched();
}

int dt_markers(const dt_world* w, int s, int f, const int* surf, const int* idx, const float* wts, int K, int M,
               const float* inv_trans, dt_fisheye cam, float* pred, float* virt, cudaStream_t stream) {
  if (!w || !surf || !idx || !wts || !inv_trans || !pred || !virt || K < 1 || M < 0 || s < 0 ||
      s >= w->n_sensors || f < 0 || f >= w->n_frames)
    return DT_ERR_ARG;
  if (M == 0) return DT_OK;
  k_markers<<<cdiv(M, NT), NT, 0, stream>>>(*w, s, f, surf, idx, wts, K, M, inv_trans, cam,
                                            reinterpret_cast<float2*>(pred), reinterpret_cast<float2*>(virt));
  return launched();
}

int dt_markers_bwd(const dt_world* w, int s, int f, const int* surf, const int* idx, const float* wts, int K, int M,
                   const float* inv_trans, dt_fisheye cam, const float* pred_b, const float* virt_b,
                   float* inv_trans_b, cudaStream_t stream) {
  if (!w || !surf || !idx || !wts || !inv_trans || K < 1 || M < 0 || s < 0 || s >= w->n_sensors || f < 0 ||
      f >= w->n_frames)
    return DT_ERR_ARG;
  if (M == 0) return DT_OK;
  k_markers_bwd<<<cdiv(M, NT), NT, 0, stream>>>(*w, s, f, surf, idx, wts, K, M, inv_trans, cam,
                                                reinterpret_cast<const float2*>(pred_b),
                                                reinterpret_cast<const float2*>(virt_b), inv_trans_b);
  return launched();
}

int dt_pose_control_vel(const dt_world* w, int s, const float* Ab, float inv_T, int f0, int nfr,
                        cudaStream_t stream) {
  if (!w || !Ab || s < 0 || s >= w->n_sensors || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames) return DT_ERR_ARG;
  k_pose_cv<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, s, Ab, inv_T, f0, nfr);
  return launched();
}

int dt_pose_control_vel_all(const dt_world* w, const float* Ab, float inv_T, int f0, int nfr, cudaStream_t stream) {
  if (!w || !Ab || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames) return DT_ERR_ARG;
  if (w->n_verts == 0) return DT_OK;
  k_pose_cv_all<<<cdiv(w->n_verts, NT), NT, 0, stream>>>(*w, Ab, inv_T, f0, nfr);
  return launched();
}

int dt_pose_control_vel_bwd(const dt_world* w, int s, const float* Ab, float inv_T, float* Ab_bar, int f0, int nfr,
                            cudaStream_t stream) {
  if (!w || !Ab || !Ab_bar || s < 0 || s >= w->n_sensors || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames)
    return DT_ERR_ARG;
  k_pose_cv_bwd<<<dim3(cdiv(w->n_verts, NT), nfr), NT, 0, stream>>>(*w, s, Ab, inv_T, Ab_bar, f0, nfr);
  return launched();
}

int dt_pose_control_vel_bwd_all(const dt_world* w, const float* Ab, float inv_T, float* Ab_bar, int f0, int nfr,
                                cudaStream_t stream) {
  if (!w || !Ab || !Ab_bar || f0 < 0 || nfr < 1 || f0 + nfr > w->n_frames) return DT_ERR_ARG;
  if (w->n_verts == 0) return DT_OK;
  k_pose_cv_bwd_all<<<dim3(cdiv(w->n_verts, NT), nfr), NT, 0, stream>>>(*w, Ab, inv_T, Ab_bar, f0, nfr);
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
