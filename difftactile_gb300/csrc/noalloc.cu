// A forward substep that allocates nothing, for callers that cannot allocate device memory.
//
// Some callers hold every device buffer they may touch in memory that another allocator owns — a
// framework's caching allocator, or an arena reserved once at start-up by a program with a fixed
// device-memory budget such as a real-time controller — and must not call cudaMalloc themselves.
// They can provide the substep's inputs and outputs (particle and FEM frames, static tables, the
// error word) but not the scratch the substep needs beyond them: the dense grid accumulator and
// velocities, the active-block flags and list, the frame's grid tape and the triangle centroids.
// dt_substep_fwd_noalloc keeps that scratch in one file-scope static device array of fixed size
// (every GPU that loads the library holds it until the process exits) and otherwise runs exactly
// dt_substep_fwd.
#include <atomic>

#include "common.cuh"

namespace {

// Capacity of the static scratch: grids up to 64^3 nodes (the reference's n_grid, 4096 blocks of
// 4x4x4), up to 8192 surface triangles.  5 node-sized float4 arrays + block lists + centroids.
constexpr size_t NA_NODES = 64 * 64 * 64;
constexpr size_t NA_BLOCKS = NA_NODES / 64;
constexpr size_t NA_TRIS = 8192;
constexpr size_t NA_OFF_ACC = 0;
constexpr size_t NA_OFF_VOUT = NA_OFF_ACC + NA_NODES;
constexpr size_t NA_OFF_TAPE_ACC = NA_OFF_VOUT + NA_NODES;
constexpr size_t NA_OFF_TAPE_VOUT = NA_OFF_TAPE_ACC + NA_NODES;
constexpr size_t NA_OFF_TAPE_CIDX = NA_OFF_TAPE_VOUT + NA_NODES;
constexpr size_t NA_OFF_FLAG = NA_OFF_TAPE_CIDX + NA_NODES;        // NA_BLOCKS ints
constexpr size_t NA_OFF_BLIST = NA_OFF_FLAG + NA_BLOCKS / 4;        // 2 * NA_BLOCKS ints
constexpr size_t NA_OFF_BCOUNT = NA_OFF_BLIST + 2 * NA_BLOCKS / 4;  // 2 ints (one float4)
constexpr size_t NA_OFF_CENT = NA_OFF_BCOUNT + 1;
constexpr size_t NA_TOTAL = NA_OFF_CENT + NA_TRIS;                   // float4 units (~21 MB)

static __device__ __align__(256) float4 g_noalloc_scratch[NA_TOTAL];

constexpr int NA_MAX_DEVICES = 64;
// The array's device address per device, looked up once (cudaGetSymbolAddress) by the first call on
// that device.  Several host threads may race to fill an entry: each stores the same address, and
// the atomic makes the store and the loads well-defined.  The address belongs to the device's
// primary context; after cudaDeviceReset the cached address is stale, so a process that resets a
// device must not call this entry point again (restart the process instead).
std::atomic<float4*> s_scratch[NA_MAX_DEVICES];

}  // namespace

extern "C" {

int dt_substep_fwd_noalloc(const dt_world* w, int f, cudaStream_t stream) {
  if (!w || f < 0 || f + 1 >= w->n_frames) return DT_ERR_ARG;
  if ((size_t)w->n_nodes > NA_NODES || (size_t)w->n_blocks > NA_BLOCKS || (size_t)w->n_tris > NA_TRIS)
    return DT_ERR_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return DT_ERR_LAUNCH;
  if (stream != nullptr) {
    // the scratch address looked up below is the current device's: a stream of another device
    // would run the kernels there against this device's address
    int sdev = -1;
    if (note_error(cudaStreamGetDevice(stream, &sdev)) != cudaSuccess) return DT_ERR_LAUNCH;
    if (sdev != dev) return DT_ERR_ARG;
  }
  float4* S = s_scratch[dev].load(std::memory_order_acquire);
  if (!S) {
    // the symbol is a host-side stand-in: its device address must be looked up per device
    void* p = nullptr;
    if (note_error(cudaGetSymbolAddress(&p, g_noalloc_scratch)) != cudaSuccess || !p) return DT_ERR_LAUNCH;
    S = static_cast<float4*>(p);
    s_scratch[dev].store(S, std::memory_order_release);
  }
  // frames f, f+1 of the caller become frames 0, 1 of a two-frame view; scratch comes from S
  dt_world v = *w;
  const size_t P = (size_t)6 * w->n_particles * 4, Vv = (size_t)w->n_verts * 4;
  v.p_state = w->p_state + (size_t)f * P;
  v.v_pos = w->v_pos + (size_t)f * Vv;
  v.v_vel = w->v_vel + (size_t)f * Vv;
  v.v_velmid = w->v_velmid + (size_t)f * Vv;
  v.v_ext = w->v_ext + (size_t)f * Vv;
  v.v_vpos = w->v_vpos + (size_t)f * Vv;
  v.v_cv = w->v_cv + (size_t)f * Vv;
  const size_t R = (size_t)w->n_rope_particles * 4;  // rope frames: state (2 planes), ext, argmin
  if (w->n_ropes > 0) {
    v.r_state = w->r_state + (size_t)f * 2 * R;
    v.r_ext = w->r_ext + (size_t)f * R;
    v.r_cidx = w->r_cidx + (size_t)f * R;
  }
  if (w->p_svd) v.p_svd = w->p_svd + (size_t)f * 6 * w->n_particles * 4;
  if (w->t_svd) v.t_svd = w->t_svd + (size_t)f * 6 * w->n_tets * 4;
  v.n_frames = 2;
  v.tape_blocks = w->n_blocks;
  v.g_acc = reinterpret_cast<float*>(S + NA_OFF_ACC);
  v.g_vout = reinterpret_cast<float*>(S + NA_OFF_VOUT);
  v.tape_acc = reinterpret_cast<float*>(S + NA_OFF_TAPE_ACC);
  v.tape_vout = reinterpret_cast<float*>(S + NA_OFF_TAPE_VOUT);
  v.tape_cidx = reinterpret_cast<int*>(S + NA_OFF_TAPE_CIDX);
  v.blk_flag = reinterpret_cast<int*>(S + NA_OFF_FLAG);
  v.tape_blist = reinterpret_cast<int*>(S + NA_OFF_BLIST);
  v.tape_bcount = reinterpret_cast<int*>(S + NA_OFF_BCOUNT);
  v.tri_cent = reinterpret_cast<float*>(S + NA_OFF_CENT);
  // the scratch keeps the previous call's contents: clear what the substep expects to start at zero
  if (note_error(cudaMemsetAsync(v.g_acc, 0, (size_t)w->n_nodes * sizeof(float4), stream)) != cudaSuccess ||
      note_error(cudaMemsetAsync(v.blk_flag, 0, (size_t)w->n_blocks * sizeof(int), stream)) != cudaSuccess ||
      note_error(cudaMemsetAsync(v.tape_bcount, 0, 2 * sizeof(int), stream)) != cudaSuccess)
    return DT_ERR_LAUNCH;
  return dt_substep_fwd(&v, 0, stream);
}

}  // extern "C"
