// Re-binning of the particles by grid cell over a rollout.
//
// Particles are sorted by cell at construction, so that consecutive particles share a base cell and
// the warp-segmented scatters of P2G and of the G2P adjoint merge them before their REDs.  As the
// material moves these runs break up (over a 1,000-step grasp the mean same-cell run in a warp falls
// from 6.4 to 1.8 particles).  dt_rebin sorts the particles of one frame by the grid node of their
// base cell again — a counting sort over the node index: keys and an atomic histogram, an exclusive
// scan of the histogram, atomic placement, then each cell's slots put back in old-slot order so that
// the result does not depend on the order of the atomics — and permutes that frame's state and the
// per-particle material index with it.  dt_rebin_permute applies a stored permutation, or its
// inverse, to the material index and to a particle adjoint buffer: the backward sweep of a
// checkpointed rollout crosses a re-binning by mapping the adjoint back to the previous order.
#include "common.cuh"

namespace {

constexpr int RB_NT = 256;
constexpr int SC_NT = 1024;                 // scan CTA
constexpr int SC_PER = 4;                   // consecutive elements per scan thread
constexpr int SC_TILE = SC_NT * SC_PER;
constexpr int RB_CELL_SORT_MAX = 256;       // cells holding more particles keep the atomics' order

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

struct Scratch {
  int* cnt;    // [n_nodes + 1] histogram, then exclusive starts, then cell ends
  int* key;    // [n_particles] base node of each particle
  int* tsum;   // [scan tiles]
  float4* tmp; // [6][n_particles] gathered record
  int* mtmp;   // [n_particles] gathered material index
};

size_t n_tiles(const dt_world* w) { return ((size_t)w->n_nodes + 1 + SC_TILE - 1) / SC_TILE; }

size_t scratch_bytes(const dt_world* w) {
  const size_t N = (size_t)w->n_particles;
  return al256(((size_t)w->n_nodes + 1) * 4) + al256(N * 4) + al256(n_tiles(w) * 4) + al256(N * 6 * 16) +
         al256(N * 4);
}

Scratch carve(const dt_world* w, void* base) {
  const size_t N = (size_t)w->n_particles;
  char* p = static_cast<char*>(base);
  Scratch s;
  s.cnt = reinterpret_cast<int*>(p);
  p += al256(((size_t)w->n_nodes + 1) * 4);
  s.key = reinterpret_cast<int*>(p);
  p += al256(N * 4);
  s.tsum = reinterpret_cast<int*>(p);
  p += al256(n_tiles(w) * 4);
  s.tmp = reinterpret_cast<float4*>(p);
  p += al256(N * 6 * 16);
  s.mtmp = reinterpret_cast<int*>(p);
  return s;
}

// inclusive scan of one value per thread over a CTA of SC_NT threads
__device__ int block_inclusive_scan(int v, int* warp_tot) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) warp_tot[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int t = lane < SC_NT / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    if (lane < SC_NT / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  const int r = v + (wid ? warp_tot[wid - 1] : 0);
  __syncthreads();  // warp_tot is reused by the next call
  return r;
}

__global__ void __launch_bounds__(RB_NT) k_rebin_key(dt_world w, int f, int* cnt, int* key) {
  pdl_entry();
  const int i = blockIdx.x * RB_NT + threadIdx.x;
  if (i >= w.n_particles) return;
  const dt_env& E = w.envs[w.p_env[i]];
  const float4 a = pplane(w, f, 0)[i];
  const float xs[3] = {a.x, a.y, a.z};
  int c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    // the base cell of the B-spline stencil, clamped into the grid (fmaxf maps NaN to 0)
    const float g = floorf(xs[d] * E.inv_dx - 0.5f);
    c[d] = (int)fminf(fmaxf(g, 0.f), (float)(E.n[d] - 1));
  }
  const int k = node_index(E, c[0], c[1], c[2]);
  key[i] = k;
  atomicAdd(cnt + k, 1);
}

// per-tile sums of data[0, n)
__global__ void __launch_bounds__(SC_NT) k_scan_reduce(const int* data, int n, int* tsum) {
  pdl_entry();
  __shared__ int warp_tot[SC_NT / 32];
  const int i0 = blockIdx.x * SC_TILE + threadIdx.x * SC_PER;
  int s = 0;
#pragma unroll
  for (int r = 0; r < SC_PER; ++r)
    if (i0 + r < n) s += data[i0 + r];
  s = block_inclusive_scan(s, warp_tot);
  if (threadIdx.x == SC_NT - 1) tsum[blockIdx.x] = s;
}

// exclusive scan of the tile sums in place, one CTA
__global__ void __launch_bounds__(SC_NT) k_scan_tiles(int* tsum, int nt) {
  pdl_entry();
  __shared__ int warp_tot[SC_NT / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b = 0; b < nt; b += SC_NT) {
    const int i = b + threadIdx.x;
    const int v = i < nt ? tsum[i] : 0;
    const int incl = block_inclusive_scan(v, warp_tot);
    const int c = carry;
    if (i < nt) tsum[i] = c + incl - v;
    __syncthreads();
    if (threadIdx.x == SC_NT - 1) carry = c + incl;
    __syncthreads();
  }
}

// exclusive scan of data[0, n) in place, each tile offset by its scanned tile sum
__global__ void __launch_bounds__(SC_NT) k_scan_apply(int* data, int n, const int* toff) {
  pdl_entry();
  __shared__ int warp_tot[SC_NT / 32];
  const int i0 = blockIdx.x * SC_TILE + threadIdx.x * SC_PER;
  int v[SC_PER], s = 0;
#pragma unroll
  for (int r = 0; r < SC_PER; ++r) {
    v[r] = i0 + r < n ? data[i0 + r] : 0;
    s += v[r];
  }
  int run = block_inclusive_scan(s, warp_tot) - s + toff[blockIdx.x];
#pragma unroll
  for (int r = 0; r < SC_PER; ++r) {
    if (i0 + r < n) data[i0 + r] = run;
    run += v[r];
  }
}

// slot of each particle: the next free slot of its cell
__global__ void __launch_bounds__(RB_NT) k_rebin_place(int n, const int* key, int* cursor, int* src) {
  pdl_entry();
  const int i = blockIdx.x * RB_NT + threadIdx.x;
  if (i < n) src[atomicAdd(cursor + key[i], 1)] = i;
}

// each cell's slots [end of the previous cell, end of this one) sorted by old slot
__global__ void __launch_bounds__(RB_NT) k_rebin_order(int n_nodes, const int* cell_end, int* src) {
  pdl_entry();
  const int k = blockIdx.x * RB_NT + threadIdx.x;
  if (k >= n_nodes) return;
  const int b = k ? cell_end[k - 1] : 0, e = cell_end[k];
  if (e - b < 2 || e - b > RB_CELL_SORT_MAX) return;
  for (int j = b + 1; j < e; ++j) {
    const int v = src[j];
    int m = j - 1;
    while (m >= b && src[m] > v) {
      src[m + 1] = src[m];
      --m;
    }
    src[m + 1] = v;
  }
}

// new slot j takes old slot src[j]: the record of frame f and the material index
__global__ void __launch_bounds__(RB_NT) k_rebin_gather(dt_world w, int f, const int* src, const int* p_mat,
                                                        float4* tmp, int* mtmp) {
  pdl_entry();
  const int j = blockIdx.x * RB_NT + threadIdx.x;
  if (j >= w.n_particles) return;
  const int o = src[j];
  const size_t N = (size_t)w.n_particles;
#pragma unroll
  for (int k = 0; k < 6; ++k) tmp[k * N + j] = pplane(w, f, k)[o];
  mtmp[j] = p_mat[o];
}

// the permutation src (new slot j <- old slot src[j]) or its inverse, on the material index and, for
// buf >= 0, on the particle adjoint buffer buf
__global__ void __launch_bounds__(RB_NT) k_rebin_permute(dt_world w, int buf, int inverse, const int* src,
                                                         const int* p_mat, float4* tmp, int* mtmp) {
  pdl_entry();
  const int j = blockIdx.x * RB_NT + threadIdx.x;
  if (j >= w.n_particles) return;
  const int o = src[j];
  const int from = inverse ? j : o, to = inverse ? o : j;
  const size_t N = (size_t)w.n_particles;
  if (buf >= 0) {
#pragma unroll
    for (int k = 0; k < 6; ++k) tmp[k * N + to] = padj(w, buf, k)[from];
  }
  mtmp[to] = p_mat[from];
}

int cdiv_i(long long a, int b) { return (int)((a + b - 1) / b); }

}  // namespace

extern "C" {

size_t dt_rebin_scratch_bytes(const dt_world* w) { return w ? scratch_bytes(w) : 0; }

int dt_rebin(const dt_world* w, int f, int* p_mat, int* src, void* scratch, cudaStream_t stream) {
  if (!w || !p_mat || !src || !scratch || f < 0 || f >= w->n_frames || !w->p_state || !w->p_env || !w->envs)
    return DT_ERR_ARG;
  if (w->n_particles <= 0) return DT_OK;
  if ((long long)w->n_nodes + 1 > 0x7fffffffLL) return DT_ERR_CAPACITY;
  const Scratch s = carve(w, scratch);
  const int N = w->n_particles, nn = w->n_nodes + 1, nt = (int)n_tiles(w);
  if (note_error(cudaMemsetAsync(s.cnt, 0, (size_t)nn * 4, stream)) != cudaSuccess) return DT_ERR_LAUNCH;
  cudaError_t e = launch_k(k_rebin_key, cdiv_i(N, RB_NT), RB_NT, 0, stream, *w, f, s.cnt, s.key);
  if (e == cudaSuccess) e = launch_k(k_scan_reduce, nt, SC_NT, 0, stream, (const int*)s.cnt, nn, s.tsum);
  if (e == cudaSuccess) e = launch_k(k_scan_tiles, 1, SC_NT, 0, stream, s.tsum, nt);
  if (e == cudaSuccess) e = launch_k(k_scan_apply, nt, SC_NT, 0, stream, s.cnt, nn, (const int*)s.tsum);
  if (e == cudaSuccess) e = launch_k(k_rebin_place, cdiv_i(N, RB_NT), RB_NT, 0, stream, N, (const int*)s.key, s.cnt, src);
  if (e == cudaSuccess)
    e = launch_k(k_rebin_order, cdiv_i(w->n_nodes, RB_NT), RB_NT, 0, stream, w->n_nodes, (const int*)s.cnt, src);
  if (e == cudaSuccess)
    e = launch_k(k_rebin_gather, cdiv_i(N, RB_NT), RB_NT, 0, stream, *w, f, (const int*)src, (const int*)p_mat, s.tmp,
                 s.mtmp);
  if (e != cudaSuccess) return DT_ERR_LAUNCH;
  float* frame = w->p_state + (size_t)f * 6 * N * 4;
  if (note_error(cudaMemcpyAsync(frame, s.tmp, (size_t)6 * N * 16, cudaMemcpyDeviceToDevice, stream)) != cudaSuccess ||
      note_error(cudaMemcpyAsync(p_mat, s.mtmp, (size_t)N * 4, cudaMemcpyDeviceToDevice, stream)) != cudaSuccess)
    return DT_ERR_LAUNCH;
  return DT_OK;
}

int dt_rebin_permute(const dt_world* w, int buf, int inverse, int* p_mat, const int* src, void* scratch,
                     cudaStream_t stream) {
  if (!w || !p_mat || !src || !scratch || buf < -1 || buf > 1 || (buf >= 0 && !w->p_adj)) return DT_ERR_ARG;
  if (w->n_particles <= 0) return DT_OK;
  const Scratch s = carve(w, scratch);
  const int N = w->n_particles;
  if (launch_k(k_rebin_permute, cdiv_i(N, RB_NT), RB_NT, 0, stream, *w, buf, inverse ? 1 : 0, src, (const int*)p_mat,
               s.tmp, s.mtmp) != cudaSuccess)
    return DT_ERR_LAUNCH;
  if (buf >= 0 && note_error(cudaMemcpyAsync(w->p_adj + (size_t)buf * 6 * N * 4, s.tmp, (size_t)6 * N * 16,
                                             cudaMemcpyDeviceToDevice, stream)) != cudaSuccess)
    return DT_ERR_LAUNCH;
  if (note_error(cudaMemcpyAsync(p_mat, s.mtmp, (size_t)N * 4, cudaMemcpyDeviceToDevice, stream)) != cudaSuccess)
    return DT_ERR_LAUNCH;
  return DT_OK;
}

}  // extern "C"
