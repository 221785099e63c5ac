// C-ABI support entry points: introspection, step set-up, frame copies, adjoint clears and the
// centre-of-mass readout.
#include <cstdio>

#include "common.cuh"

namespace {

constexpr int NT = 256;
inline int cdiv(int a, int b) { return (a + b - 1) / b; }
inline int launched() { return launch_status(cudaGetLastError()); }

// Contact.reset (grasp_plastic.py:386-392) equivalent for the per-step tape: frame counters to
// zero, FEM frame 0 accumulators prepared.
__global__ void k_step_begin(dt_world w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < w.n_frames) w.tape_bcount[i] = 0;
  if (i < w.n_verts) {
    vframe(w.v_velmid, w, 0)[i] = vframe(w.v_vel, w, 0)[i];
    vframe(w.v_ext, w, 0)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// compute_obj_pos (grasp_plastic.py:259-261): per-env sum of x, scaled by 1/count at the end
__global__ void k_com(dt_world w, int f, float* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= w.n_particles) return;
  const int e = __ldg(w.p_env + p);
  const dt_env& E = w.envs[e];
  const float inv = 1.f / (float)(E.p_end - E.p_begin);
  const float4 x = __ldg(pplane(w, f, 0) + p);
  // warp-aggregate when the whole warp is in one env
  const unsigned mask = __match_any_sync(0xffffffffu, e);
  float sx = x.x * inv, sy = x.y * inv, sz = x.z * inv;
  if (mask == 0xffffffffu) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(out + 4 * e + 0, sx);
      atomicAdd(out + 4 * e + 1, sy);
      atomicAdd(out + 4 * e + 2, sz);
    }
  } else {
    atomicAdd(out + 4 * e + 0, sx);
    atomicAdd(out + 4 * e + 1, sy);
    atomicAdd(out + 4 * e + 2, sz);
  }
}

__global__ void k_com_bwd(dt_world w, int f, const float* adj) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= w.n_particles) return;
  const int e = __ldg(w.p_env + p);
  const dt_env& E = w.envs[e];
  const float inv = 1.f / (float)(E.p_end - E.p_begin);
  float4* a = padj(w, f & 1, 0) + p;
  float4 v = *a;
  v.x += inv * adj[4 * e + 0];
  v.y += inv * adj[4 * e + 1];
  v.z += inv * adj[4 * e + 2];
  *a = v;
}

}  // namespace

extern "C" {

int dt_abi_version(void) { return DT_ABI_VERSION; }
size_t dt_sizeof_world(void) { return sizeof(dt_world); }
size_t dt_sizeof_env(void) { return sizeof(dt_env); }
size_t dt_sizeof_sensor(void) { return sizeof(dt_sensor); }
size_t dt_sizeof_material(void) { return sizeof(dt_material); }
size_t dt_sizeof_rope(void) { return sizeof(dt_rope); }

int dt_set_pdl(int on) {
  const int old = pdl_flag();
  pdl_flag() = on ? 1 : 0;
  return old;
}

int dt_get_pdl(void) { return pdl_flag(); }

int dt_last_error(char* buf, size_t len) {
  const cudaError_t e = last_cuda_error();
  last_cuda_error() = cudaSuccess;
  if (buf && len) snprintf(buf, len, "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
  return (int)e;
}

int dt_step_begin(const dt_world* w, cudaStream_t stream) {
  if (!w || w->n_frames < 2) return DT_ERR_ARG;
  int n = w->n_frames > w->n_verts ? w->n_frames : w->n_verts;
  k_step_begin<<<cdiv(n, NT), NT, 0, stream>>>(*w);
  return launched();
}

int dt_copy_frame(const dt_world* w, int src, int dst, cudaStream_t stream) {
  if (!w || src < 0 || dst < 0 || src >= w->n_frames || dst >= w->n_frames) return DT_ERR_ARG;
  if (src == dst) return DT_OK;
  const size_t pbytes = (size_t)6 * w->n_particles * 16;
  if (pbytes && note_error(cudaMemcpyAsync(w->p_state + (size_t)dst * 6 * w->n_particles * 4,
                                w->p_state + (size_t)src * 6 * w->n_particles * 4, pbytes, cudaMemcpyDeviceToDevice,
                                stream)) != cudaSuccess)
    return DT_ERR_LAUNCH;
  const size_t vbytes = (size_t)w->n_verts * 16;
  float* arrs[4] = {w->v_pos, w->v_vel, w->v_vpos, w->v_cv};
  for (float* a : arrs) {
    if (vbytes && note_error(cudaMemcpyAsync(a + (size_t)dst * w->n_verts * 4, a + (size_t)src * w->n_verts * 4, vbytes,
                                  cudaMemcpyDeviceToDevice, stream)) != cudaSuccess)
      return DT_ERR_LAUNCH;
  }
  // rope pos, vel, travel_info (PBDRope.copy_frame, PBD_rope.py:182-187)
  const size_t rbytes = (size_t)2 * w->n_rope_particles * 16;
  if (rbytes && note_error(cudaMemcpyAsync(w->r_state + (size_t)dst * 2 * w->n_rope_particles * 4,
                                w->r_state + (size_t)src * 2 * w->n_rope_particles * 4, rbytes,
                                cudaMemcpyDeviceToDevice, stream)) != cudaSuccess)
    return DT_ERR_LAUNCH;
  return DT_OK;
}

int dt_adj_clear(const dt_world* w, cudaStream_t stream) {
  if (!w) return DT_ERR_ARG;
  struct {
    void* p;
    size_t n;
  } z[] = {
      {w->p_adj, (size_t)2 * 6 * w->n_particles * 16},
      {w->g_adj_vout, (size_t)w->n_nodes * 16},
      {w->g_adj_acc, (size_t)w->n_nodes * 16},
      {w->v_adj_pos, (size_t)2 * w->n_verts * 16},
      {w->v_adj_vel, (size_t)2 * w->n_verts * 16},
      {w->v_adj_vpos, (size_t)2 * w->n_verts * 16},
      {w->v_adj_velmid, (size_t)w->n_verts * 16},
      {w->v_adj_ext, (size_t)w->n_verts * 16},
      {w->v_adj_cv, (size_t)w->n_frames * w->n_verts * 16},
      {w->mat_adj, (size_t)w->n_materials * 16},
      {w->r_adj, (size_t)4 * w->n_rope_particles * 16},
      {w->r_extb, (size_t)w->n_rope_particles * 16},
  };
  for (auto& e : z)
    if (e.p && e.n && note_error(cudaMemsetAsync(e.p, 0, e.n, stream)) != cudaSuccess) return DT_ERR_LAUNCH;
  return DT_OK;
}

int dt_com(const dt_world* w, int f, float* out, cudaStream_t stream) {
  if (!w || !out || f < 0 || f >= w->n_frames) return DT_ERR_ARG;
  if (note_error(cudaMemsetAsync(out, 0, (size_t)w->n_envs * 16, stream)) != cudaSuccess) return DT_ERR_LAUNCH;
  if (w->n_particles == 0) return DT_OK;
  k_com<<<cdiv(w->n_particles, NT), NT, 0, stream>>>(*w, f, out);
  return launched();
}

int dt_com_bwd(const dt_world* w, int f, const float* adj_com, cudaStream_t stream) {
  if (!w || !adj_com || f < 0 || f >= w->n_frames) return DT_ERR_ARG;
  if (w->n_particles == 0) return DT_OK;
  k_com_bwd<<<cdiv(w->n_particles, NT), NT, 0, stream>>>(*w, f, adj_com);
  return launched();
}

}  // extern "C"
