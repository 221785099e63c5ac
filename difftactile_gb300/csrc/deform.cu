// Shape-target (deform) loss of an environment's object, tasks/deform_loss.py:8-146:
//   grid mass   compute_grid_m_kernel, object_model/mpm_plastic.py:169-178 — mass-only P2G of frame f
//               (quadratic B-spline weights, node i at i dx) into an [n_nodes] array in the world's
//               block layout;
//   loss        density_loss = sum_I |m_I - target_I|, sdf_loss = sum_I sdf_I m_I,
//               loss += w_density density_loss + w_sdf sdf_loss (compute_*_loss_kernel,
//               sum_up_loss_kernel);
//   adjoint     d loss / d m_I = w_density sign(m_I - target_I) + w_sdf sdf_I, scattered back to the
//               particle positions through the weight gradients (compute_grid_m_kernel.grad);
//   target SDF  update_target_sdf: 2 n passes of nearest-point propagation over offsets in
//               [-3, 3)^3 \ {0}, distance norm(eps 1e-8), seeded where target > 1e-4.
// Grids use the world's block layout (node_index of the env); values of nodes outside the env's
// n^3 (block padding) stay zero.
#include "common.cuh"

namespace {

constexpr int NT = 256;
inline int cdiv(int a, int b) { return (a + b - 1) / b; }

DT_DEV bool env_node(const dt_env& E, int local, int& i, int& j, int& k) {
  const int lb = local >> 6, l = local & 63;
  const int bk = lb % E.nb[2], bj = (lb / E.nb[2]) % E.nb[1], bi = lb / (E.nb[1] * E.nb[2]);
  i = 4 * bi + (l >> 4);
  j = 4 * bj + ((l >> 2) & 3);
  k = 4 * bk + (l & 3);
  return i < E.n[0] && j < E.n[1] && k < E.n[2];
}

// B-spline weights w[o][d] and their derivatives (d/dfx) for the mass P2G (node i at i dx)
DT_DEV bool mass_base(const dt_env& E, v3 x, int base[3], float w[3][3], float dw[3][3]) {
  const float xc[3] = {x.x, x.y, x.z};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    base[d] = (int)(xc[d] * E.inv_dx - 0.5f);  // cast(int) truncates toward zero, as the reference
    const float fx = xc[d] * E.inv_dx - (float)base[d];
    w[0][d] = 0.5f * (1.5f - fx) * (1.5f - fx);
    w[1][d] = 0.75f - (fx - 1.f) * (fx - 1.f);
    w[2][d] = 0.5f * (fx - 0.5f) * (fx - 0.5f);
    dw[0][d] = fx - 1.5f;
    dw[1][d] = -2.f * (fx - 1.f);
    dw[2][d] = fx - 0.5f;
    if (base[d] < 0 || base[d] + 2 >= E.n[d]) return false;
  }
  return true;
}

__global__ void k_grid_mass(dt_world w, int e, int f, float* m) {
  const dt_env& E = w.envs[e];
  const int p = E.p_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= E.p_end) return;
  const v3 x = f4to3(__ldg(pplane(w, f, 0) + p));
  int base[3];
  float wt[3][3], dw[3][3];
  if (!mass_base(E, x, base, wt, dw)) {
    set_err(w, DT_DEVERR_PARTICLE_OOB);
    return;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        atomicAdd(m + node_index(E, base[0] + a, base[1] + b, base[2] + c), (wt[a][0] * wt[b][1]) * wt[c][2] * E.p_mass);
}

__global__ void k_deform_loss(dt_world w, int e, const float* __restrict__ m, const float* __restrict__ tgt,
                              const float* __restrict__ sdf, float wd, float ws, float* loss) {
  __shared__ float red[NT / 32];
  const dt_env& E = w.envs[e];
  const int local = blockIdx.x * blockDim.x + threadIdx.x;
  const int nn = 64 * E.nb[0] * E.nb[1] * E.nb[2];
  float v = 0.f;
  int i, j, k;
  if (local < nn && env_node(E, local, i, j, k)) {
    const int g = E.node_off + local;
    v = wd * fabsf(m[g] - tgt[g]) + ws * (sdf[g] * m[g]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int q = 0; q < NT / 32; ++q) s += red[q];
    atomicAdd(loss, s);
  }
}

__global__ void k_deform_loss_bwd(dt_world w, int e, int f, const float* __restrict__ m,
                                  const float* __restrict__ tgt, const float* __restrict__ sdf, float wd, float ws,
                                  float lb) {
  const dt_env& E = w.envs[e];
  const int p = E.p_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= E.p_end) return;
  const v3 x = f4to3(__ldg(pplane(w, f, 0) + p));
  int base[3];
  float wt[3][3], dw[3][3];
  if (!mass_base(E, x, base, wt, dw)) return;
  v3 fxb = v3{0.f, 0.f, 0.f};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int g = node_index(E, base[0] + a, base[1] + b, base[2] + c);
        const float d = m[g] - tgt[g];
        const float gm = lb * (wd * (d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f)) + ws * sdf[g]) * E.p_mass;
        fxb.x += gm * (dw[a][0] * wt[b][1] * wt[c][2]);
        fxb.y += gm * (wt[a][0] * dw[b][1] * wt[c][2]);
        fxb.z += gm * (wt[a][0] * wt[b][1] * dw[c][2]);
      }
  // x adjoint of frame f: plane 0 .xyz of the double-buffered particle adjoint
  float4* ax = reinterpret_cast<float4*>(w.p_adj) + (size_t)(f & 1) * 6 * w.n_particles + p;
  float4 a0 = *ax;
  a0.x += E.inv_dx * fxb.x;
  a0.y += E.inv_dx * fxb.y;
  a0.z += E.inv_dx * fxb.z;
  *ax = a0;
}

// one propagation pass: nearest seed point of every node from its neighbours' of the previous pass
__global__ void k_sdf_pass(dt_world w, int e, const float* __restrict__ tgt, const float4* __restrict__ prev,
                           float4* next) {
  const dt_env& E = w.envs[e];
  const int local = blockIdx.x * blockDim.x + threadIdx.x;
  const int nn = 64 * E.nb[0] * E.nb[1] * E.nb[2];
  if (local >= nn) return;
  int i, j, k;
  const int g = E.node_off + local;
  if (!env_node(E, local, i, j, k)) {
    next[g] = make_float4(0.f, 0.f, 0.f, 1000.f);
    return;
  }
  const v3 gp = v3{(float)i * E.dx, (float)j * E.dx, (float)k * E.dx};
  if (tgt[g] > 1e-4f) {
    next[g] = v3to4(gp, 0.f);
    return;
  }
  float best = 1000.f;
  v3 bp = v3{0.f, 0.f, 0.f};
  for (int a = -3; a < 3; ++a)
    for (int b = -3; b < 3; ++b)
      for (int c = -3; c < 3; ++c) {
        if (a == 0 && b == 0 && c == 0) continue;
        const int vi = i + a, vj = j + b, vk = k + c;
        if (vi < 0 || vj < 0 || vk < 0 || vi >= E.n[0] || vj >= E.n[1] || vk >= E.n[2]) continue;
        const float4 q = prev[node_index(E, vi, vj, vk)];
        if (!(q.w < 1000.f)) continue;
        const v3 dq = gp - f4to3(q);
        const float dist = sqrtf(dot(dq, dq) + 1e-8f);
        if (dist < best) {
          best = dist;
          bp = f4to3(q);
        }
      }
  next[g] = v3to4(bp, best);
}

__global__ void k_sdf_out(dt_world w, int e, const float4* __restrict__ src, float* sdf) {
  const dt_env& E = w.envs[e];
  const int local = blockIdx.x * blockDim.x + threadIdx.x;
  const int nn = 64 * E.nb[0] * E.nb[1] * E.nb[2];
  if (local >= nn) return;
  int i, j, k;
  const int g = E.node_off + local;
  sdf[g] = env_node(E, local, i, j, k) ? src[g].w : 0.f;
}

__global__ void k_sdf_init(dt_world w, int e, float4* buf) {
  const dt_env& E = w.envs[e];
  const int local = blockIdx.x * blockDim.x + threadIdx.x;
  const int nn = 64 * E.nb[0] * E.nb[1] * E.nb[2];
  if (local < nn) buf[E.node_off + local] = make_float4(0.f, 0.f, 0.f, 1000.f);
}

inline int launched() { return launch_status(cudaGetLastError()); }

}  // namespace

extern "C" {

int dt_grid_mass(const dt_world* w, int e, int f, float* m, cudaStream_t stream) {
  if (!w || !m || e < 0 || e >= w->n_envs || f < 0 || f >= w->n_frames) return DT_ERR_ARG;
  k_grid_mass<<<cdiv(w->n_particles > 0 ? w->n_particles : 1, NT), NT, 0, stream>>>(*w, e, f, m);
  return launched();
}

int dt_deform_loss(const dt_world* w, int e, const float* m, const float* target, const float* sdf, float w_density,
                   float w_sdf, float* loss, cudaStream_t stream) {
  if (!w || !m || !target || !sdf || !loss || e < 0 || e >= w->n_envs) return DT_ERR_ARG;
  k_deform_loss<<<cdiv(w->n_nodes, NT), NT, 0, stream>>>(*w, e, m, target, sdf, w_density, w_sdf, loss);
  return launched();
}

int dt_deform_loss_bwd(const dt_world* w, int e, int f, const float* m, const float* target, const float* sdf,
                       float w_density, float w_sdf, float loss_bar, cudaStream_t stream) {
  if (!w || !m || !target || !sdf || e < 0 || e >= w->n_envs || f < 0 || f >= w->n_frames) return DT_ERR_ARG;
  k_deform_loss_bwd<<<cdiv(w->n_particles > 0 ? w->n_particles : 1, NT), NT, 0, stream>>>(*w, e, f, m, target, sdf,
                                                                                          w_density, w_sdf, loss_bar);
  return launched();
}

int dt_target_sdf(const dt_world* w, int e, const float* target, float* sdf, float* scratch, int passes,
                  cudaStream_t stream) {
  if (!w || !target || !sdf || !scratch || e < 0 || e >= w->n_envs || passes < 1) return DT_ERR_ARG;
  float4* a = reinterpret_cast<float4*>(scratch);
  float4* b = a + w->n_nodes;
  const int nb = cdiv(w->n_nodes, NT);
  k_sdf_init<<<nb, NT, 0, stream>>>(*w, e, a);
  for (int it = 0; it < passes; ++it) {
    k_sdf_pass<<<nb, NT, 0, stream>>>(*w, e, target, a, b);
    float4* t = a;
    a = b;
    b = t;
  }
  k_sdf_out<<<nb, NT, 0, stream>>>(*w, e, a, sdf);
  return launched();
}

}  // extern "C"
