// Forward substep kernels (sm_103a).
//
// One substep f -> f+1 of the coupled MPM object + FEM sensors, in three launches:
//   L1 k_fwd_p2g_fem : particles  — compute_new_F, 3x3 SVD, return map, stress, P2G scatter
//                      (mpm_elastic.py:135-208, mpm_plastic.py:151-256, multi_obj.py:228-252);
//                      tets       — FEM elastic forces into vel (fem_sensor.py:409-440);
//                      triangles  — surface-triangle centroids for the contact argmin.
//   L2 k_fwd_grid    : active grid blocks — occupancy, argmin triangle, SDF, penalty/friction
//                      contact, grid velocity update with walls (mpm_elastic.py:211-240,
//                      grasp_plastic.py:205-216,270-299, fem_sensor.py:344-406); writes the
//                      per-frame grid tape and clears the P2G accumulator.
//   L3 k_fwd_g2p_fem : particles  — G2P gather, APIC C, advection (mpm_elastic.py:244-260);
//                      vertices   — FEM integration with the driven base layer
//                      (fem_sensor.py:444-457, gripper_fem.py:404-418).
//
// P2G scatter: a CTA takes 128 consecutive particles (kept spatially sorted by the host); with
// DT_SCATTER_TILE their stencil records are gathered per node of the chunk's bounding box in shared
// memory and flushed with one 16-byte vector RED per node (common.cuh: stencil_scatter), with
// DT_SCATTER_GLOBAL each particle issues its 27 vector REDs directly.
#include "contact.cuh"
#include <climits>

namespace {

constexpr int NT_TILE = 128;      // threads per CTA of the particle roles with the TILE scatter
constexpr int TILE_MAX = 1728;    // shared P2G tile capacity in nodes (12^3), 27 KB of float4
// lanes per node in the grid kernel's contact search (dt_world.contact_lanes): 8 (shorter chains,
// for launches with few active blocks) or 4 (fewer issued instructions per node); a CTA of
// 64 * lanes threads takes its blocks four at a time.  Two lanes per node measured slower on the
// population (grid kernel 201 -> 267 us: each lane's chain twice as long, and its 16 cached group
// distances spill)
constexpr int SMEM_CENT_MAX = 12288;  // triangle centroids staged in shared memory (192 KB)

__device__ void mark_block(const dt_world& w, int f, int b) {
  volatile int* fl = w.blk_flag + b;
  if (*fl == 0 && atomicExch(w.blk_flag + b, 1) == 0) {
    int s = atomicAdd(w.tape_bcount + f, 1);
    if (s < w.n_blocks) w.tape_blist[(size_t)f * w.n_blocks + s] = b;
  }
}

// P2G of one CTA's particles (mpm_elastic.py:176-208 / mpm_plastic.py:222-256 / multi_obj.py:228-252):
// contribution at node base + o is W_o (p_mass v + A (o - fx) dx) = W_o (b + (o - 1) . (dx A)), with
// A = stress + p_mass C and b = p_mass v + A (1 - fx) dx (the middle node's) precomputed once per particle.
template <int MODE, int NT>
__device__ void p2g_chunk(const dt_world& w, int f, int chunk, float4* tile, int* sh) {
  const int p = chunk * NT + threadIdx.x;
  const bool valid = p < w.n_particles;
  PRec r;
  Stress s;
  int base[3] = {0, 0, 0};
  float fx[3] = {0.f, 0.f, 0.f};
  bool ok = false;
  int env = 0;
  float wx[3] = {0.f, 0.f, 0.f}, wy[3] = {0.f, 0.f, 0.f}, wz[3] = {0.f, 0.f, 0.f};
  v3 b = v3{0.f, 0.f, 0.f}, c0 = b, c1 = b, c2 = b;
  float pm = 0.f;
  if (valid) {
    float4 q[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) q[k] = ldg4(pplane(w, f, k) + p);
    unpack_rec(q, r);
    env = __ldg(w.p_env + p);
    const dt_env& E = w.envs[env];
    ok = particle_base(E, r.x, base, fx);
    if (!ok) set_err(w, DT_DEVERR_PARTICLE_OOB);
    if (ok) {
      const dt_material M = w.materials[__ldg(w.p_mat + p)];
      constitutive(r.C, r.F, w.dt, M, w.svd_sweeps, s);
      if (w.p_svd && !w.skip_tape && M.model != DT_MODEL_NEOHOOKEAN)
        store_svd(w, f, p, s.U, s.sig, s.V, s.yield);  // for the adjoint
      pm = E.p_mass;
      const float dx = E.dx, sk = E.stress_k;
      m3 A;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) A.a[i][j] = sk * s.cauchy.a[i][j] + pm * r.C.a[i][j];
      c0 = dx * mcol(A, 0);
      c1 = dx * mcol(A, 1);
      c2 = dx * mcol(A, 2);
      // the affine momentum at the middle node of the stencil, (1 - fx) dx from the particle
      b = pm * r.v + mvec(A, v3{(1.f - fx[0]) * dx, (1.f - fx[1]) * dx, (1.f - fx[2]) * dx});
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        wx[i] = bsw(i, fx[0]);
        wy[i] = bsw(i, fx[1]);
        wz[i] = bsw(i, fx[2]);
      }
    } else {
      s.Fp = r.F;
    }
    // F[f+1] (mpm_elastic.py:208); plane 3 is shared with C, which G2P writes
    reinterpret_cast<float*>(pplane(w, f + 1, 3) + p)[3] = s.Fp.a[0][0];
    pplane(w, f + 1, 4)[p] = make_float4(s.Fp.a[0][1], s.Fp.a[0][2], s.Fp.a[1][0], s.Fp.a[1][1]);
    pplane(w, f + 1, 5)[p] = make_float4(s.Fp.a[1][2], s.Fp.a[2][0], s.Fp.a[2][1], s.Fp.a[2][2]);
  }
  StencilRec rec;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    rec.wx[i] = wx[i];
    rec.wy[i] = wy[i];
    rec.wz[i] = wz[i];
  }
  rec.q = make_float4(b.x, b.y, b.z, pm);
  rec.c0 = c0;
  rec.c1 = c1;
  rec.c2 = c2;
  // the blocks of the node box [l, h], shared out as i = start, start + stride, ...
  auto mark_box = [&](const dt_env& E0, int l0, int l1, int l2, int h0, int h1, int h2, int start, int stride) {
    const int b0 = l0 >> 2, b1 = l1 >> 2, b2 = l2 >> 2;
    const int n0 = (h0 >> 2) - b0 + 1, n1 = (h1 >> 2) - b1 + 1, n2 = (h2 >> 2) - b2 + 1;
    for (int i = start; i < n0 * n1 * n2; i += stride) {
      const int c = i % n2, bb = (i / n2) % n1, a = i / (n1 * n2);
      mark_block(w, f, block_index(E0, b0 + a, b1 + bb, b2 + c));
    }
  };
  auto mark_one = [&](const dt_env& E) {
    for (int t = 0; t < 8; ++t) {
      const int bi = (base[0] + 2 * (t >> 2)) >> 2, bj = (base[1] + 2 * ((t >> 1) & 1)) >> 2,
                bk = (base[2] + 2 * (t & 1)) >> 2;
      mark_block(w, f, block_index(E, bi, bj, bk));
    }
  };
  stencil_scatter<NT, TILE_MAX, MODE>(w, chunk, ok, env, base, rec, reinterpret_cast<float*>(tile), sh,
                                      reinterpret_cast<float4*>(w.g_acc), mark_box, mark_one);
}

// FEM elastic forces of one tet (fem_sensor.py:409-440): the reference's stable-Neo-Hookean-like P with
// current volume weighting, or linear corotated with rest volume (dt_sensor.model); velocity increments
// accumulated into velmid[f] with vector REDs
__device__ void fem_tet(const dt_world& w, int f, int t) {
  const int4 tv = __ldg(reinterpret_cast<const int4*>(w.tets) + t);
  const dt_sensor& S = w.sensors[__ldg(w.tet_sensor + t)];
  const float4* Bp = reinterpret_cast<const float4*>(w.tet_B) + 3 * (size_t)t;
  m3 B;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float4 row = __ldg(Bp + r);
    B.a[r][0] = row.x;
    B.a[r][1] = row.y;
    B.a[r][2] = row.z;
  }
  const float4* P = vframe(w.v_pos, w, f);
  v3 a = f4to3(P[tv.x]), b = f4to3(P[tv.y]), c = f4to3(P[tv.z]), d = f4to3(P[tv.w]);
  m3 D;
  v3 cols[3] = {a - d, b - d, c - d};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    D.a[0][k] = cols[k].x;
    D.a[1][k] = cols[k].y;
    D.a[2][k] = cols[k].z;
  }
  float Vi = fabsf(mdet(D)) / 6.f;
  const m3 Fe = mmul(D, B);
  m3 Pk;
  if (S.model == DT_FEM_LINEAR_COROTATED) {
    // P = 2 mu (F - R) + lam tr(R^T F - I) R (tr(R^T F) = sum of the singular values), rest volume
    m3 U, V;
    v3 sg;
    svd3(Fe, U, sg, V, w.svd_sweeps);
    if (w.t_svd && !w.skip_tape) store_svd_of(w.t_svd, w.n_tets, f, t, U, sg, V, false);  // for the adjoint
    const m3 R = mmulT(U, V);
    const float c = ((sg.x + sg.y) + sg.z) - 3.f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Pk.a[i][j] = 2.f * S.mu * (Fe.a[i][j] - R.a[i][j]) + S.lam * c * R.a[i][j];
    Vi = 1.f / (6.f * fabsf(mdet(B)));
  } else {
    const float J = mdet(Fe);
    const float IC = mdot(Fe, Fe);
    const m3 cof = mcof(Fe);
    const float k1 = S.mu * (1.f - 1.f / (IC + 1.f));
    const float k2 = S.lam * (J - S.alpha);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Pk.a[i][j] = k1 * Fe.a[i][j] + k2 * cof.a[i][j];
  }
  const m3 H = mmulT(Pk, B);  // P B^T
  const float s = -Vi * S.dt_over_m;
  float4* VM = vframe(w.v_velmid, w, f);
  v3 h0 = s * mcol(H, 0), h1 = s * mcol(H, 1), h2 = s * mcol(H, 2);
  red_add_v4(VM + tv.x, v3to4(h0));
  red_add_v4(VM + tv.y, v3to4(h1));
  red_add_v4(VM + tv.z, v3to4(h2));
  red_add_v4(VM + tv.w, v3to4(-((h0 + h1) + h2)));
}

// centroid of the triangle at contact-search position t, tagged with its sensor-local index
__device__ void tri_centroid(const dt_world& w, int f, int t) {
  const int src = w.tri_perm ? __ldg(w.tri_perm + t) : t;
  const int4 tr = __ldg(reinterpret_cast<const int4*>(w.tris) + src);
  const dt_sensor& S = w.sensors[tr.w];
  const float4* P = vframe(w.v_pos, w, f);
  float4 a = P[tr.x], b = P[tr.y], c = P[tr.z];
  const float third = 1.f / 3.f;
  float4 o;
  o.x = __fmul_rn(third, __fadd_rn(__fadd_rn(a.x, b.x), c.x));
  o.y = __fmul_rn(third, __fadd_rn(__fadd_rn(a.y, b.y), c.y));
  o.z = __fmul_rn(third, __fadd_rn(__fadd_rn(a.z, b.z), c.z));
  o.w = __int_as_float(src - S.f_off);
  reinterpret_cast<float4*>(w.tri_cent)[t] = o;
}

template <int MODE, int NT, int PPT>
__global__ void __launch_bounds__(NT, DT_MINB(DT_MINB_FWD_P2G, NT)) k_fwd_p2g_fem(dt_world w, int f, int nb_p, int nb_t, int nb_f) {
  pdl_entry();
  extern __shared__ float4 tile[];  // stencil records (TILE mode) or the grid tile (SMEM mode); none otherwise
  __shared__ int sh[8];
  int b = blockIdx.x;
  if (b < nb_p) {
    if (PPT == 1) {
      p2g_chunk<MODE, NT>(w, f, b, tile, sh);
    } else {
      int c0, c1;
      cta_chunks(w, NT, PPT, b, c0, c1);
      for (int c = c0; c < c1; ++c) {
        // the shared box and tile of the previous chunk (the warp scatter shares nothing between chunks)
        if (c > c0 && !(MODE >= DT_SCATTER_WARP && MODE < DT_MODE_SMEM)) __syncthreads();
        p2g_chunk<MODE, NT>(w, f, c, tile, sh);
      }
    }
    return;
  }
  b -= nb_p;
  if (b < nb_t) {
    int t = b * NT + threadIdx.x;
    if (t < w.n_tets) fem_tet(w, f, t);
    return;
  }
  b -= nb_t;
  if (b < nb_f) {
    int t = b * NT + threadIdx.x;
    if (t < w.n_tris) tri_centroid(w, f, t);
  }
}

// ---------------------------------------------------------------------------------------------
// L2: grid update + contact over the frame's active blocks.  64 x GRID_LPN threads per 4x4x4 block:
// GRID_LPN (8 or 4) lanes per node share the node's argmin over the sensor's triangle centroids
// (staged in shared memory, contact.cuh: closest_tri); the (distance, index) pairs are combined
// lexicographically, which is exactly the sequential scan's first-minimum-wins result.  Then each
// 64-thread group takes one block's nodes, one per thread, for the contact force and the grid update,
// so the serial per-node work issues from 2 warps per block instead of from one lane in GRID_LPN of
// every warp.
// ---------------------------------------------------------------------------------------------
// CAND: sensors of more than 32 groups of centroids are searched over per-block candidate groups
template <int GRID_LPN, bool CAND, int GRID_NT = 64 * GRID_LPN>
__global__ void __launch_bounds__(GRID_NT, DT_MINB_FWD_GRID * 1024 / GRID_NT / 4) k_fwd_grid(dt_world w, int f, int smem_cap) {
  pdl_entry();
  extern __shared__ float4 scent[];
  float4* gbox = scent + smem_cap;  // 2 float4 per group of 32 centroids
  // The CTA takes its run of the active list KB blocks at a time: all lanes search the KB blocks one
  // after the other, then each 64-thread group runs one block's node pass.  The argmins of every node
  // per sensor slot are double-buffered over these steps: the search of the next KB blocks fills one
  // buffer while the node passes of the previous ones read the other.
  constexpr int KB = GRID_NT / 64 < 4 ? GRID_NT / 64 : 4;
  __shared__ int s_cid[2][KB][DT_MAX_SENSORS_PER_ENV][64];
  __shared__ int s_cand[CAND ? SMEM_CENT_MAX / 32 : 1];  // candidate groups of the block
  __shared__ int s_csh[2];
  const int cnt = *((volatile int*)(w.tape_bcount + f));
  const int tid = threadIdx.x;
  const int l = tid / GRID_LPN, sub = tid % GRID_LPN;
  const float third = 1.f / 3.f;
  float4* acc = reinterpret_cast<float4*>(w.g_acc);
  float4* vout = reinterpret_cast<float4*>(w.g_vout);
  const float4* P = vframe(w.v_pos, w, f);
  const float4* VM = vframe(w.v_velmid, w, f);
  float4* EXT = vframe(w.v_ext, w, f);
  const int4* tris = reinterpret_cast<const int4*>(w.tris);
  int staged = -1;
  // a contiguous run of the active list per CTA: blocks of one environment sit together in the list
  // (they are marked by the P2G CTAs of that environment's particles), so the CTA restages the
  // sensor's centroids only when its run crosses into another environment
  const int per = (cnt + (int)gridDim.x - 1) / (int)gridDim.x;
  const int e_end = min(cnt, ((int)blockIdx.x + 1) * per);
  int it = 0;
  for (int e0 = blockIdx.x * per; e0 < e_end; e0 += KB, it ^= 1) {
    const int nk = min(KB, e_end - e0);  // blocks in this step (CTA-uniform)
    // ---- search: GRID_LPN lanes per node, block after block ----
    for (int h = 0; h < nk; ++h) {
      const int b = w.tape_blist[(size_t)f * w.n_blocks + e0 + h];
      const dt_env& E = w.envs[__ldg(w.blk_env + b)];
      const int lb = b - E.blk_off;
      const int bk = lb % E.nb[2], bj = (lb / E.nb[2]) % E.nb[1], bi = lb / (E.nb[1] * E.nb[2]);
      const int i = 4 * bi + (l >> 4), j = 4 * bj + ((l >> 2) & 3), k = 4 * bk + (l & 3);
      const bool occ = acc[E.node_off + (lb << 6) + l].w > E.eps;  // check_grid_occupy, mpm_elastic.py:213
      const float px = __fmul_rn(__fadd_rn((float)i, 0.5f), E.dx), py = __fmul_rn(__fadd_rn((float)j, 0.5f), E.dx),
                  pz = __fmul_rn(__fadd_rn((float)k, 0.5f), E.dx);
#pragma unroll
      for (int q = 0; q < DT_MAX_SENSORS_PER_ENV; ++q) {
        const int si = E.s_begin + q;  // block-uniform
        if (si >= E.s_end) break;
        const dt_sensor& S = w.sensors[si];
        const bool in_smem = S.nf <= smem_cap;
        if (in_smem && staged != si) {  // block-uniform
          stage_sensor<GRID_NT>(w, S, scent, gbox);
          staged = si;
        }
        const int Gall = (S.nf + 31) >> 5;
        int nc = 0;
        const int* cand = nullptr;
        if (CAND && in_smem && Gall > DT_CAND_MIN_GROUPS) {  // block-uniform: the groups any node of this block can need
          const float4 qlo = make_float4(__fmul_rn(__fadd_rn((float)(4 * bi), 0.5f), E.dx),
                                         __fmul_rn(__fadd_rn((float)(4 * bj), 0.5f), E.dx),
                                         __fmul_rn(__fadd_rn((float)(4 * bk), 0.5f), E.dx), 0.f);
          const float4 qhi = make_float4(__fmul_rn(__fadd_rn((float)(4 * bi + 3), 0.5f), E.dx),
                                         __fmul_rn(__fadd_rn((float)(4 * bj + 3), 0.5f), E.dx),
                                         __fmul_rn(__fadd_rn((float)(4 * bk + 3), 0.5f), E.dx), 0.f);
          nc = block_candidates<GRID_NT>(gbox, Gall, qlo, qhi, s_cand, s_csh);
          cand = s_cand;
        }
        const int kk = closest_tri<GRID_LPN>(w, S, scent, gbox, in_smem, occ, px, py, pz, sub, cand, nc);
        if (sub == 0) s_cid[it][h][q][l] = kk;
      }
    }
    __syncthreads();
    // ---- node passes: one thread per node, 64-thread group h for block h of the step ----
    const int h = tid >> 6, nd = tid & 63;
    if (h >= nk) continue;
    const int e = e0 + h;
    const int b = w.tape_blist[(size_t)f * w.n_blocks + e];
    const dt_env& E = w.envs[__ldg(w.blk_env + b)];
    const int lb = b - E.blk_off;
    const int bk = lb % E.nb[2], bj = (lb / E.nb[2]) % E.nb[1], bi = lb / (E.nb[1] * E.nb[2]);
    const int i = 4 * bi + (nd >> 4), j = 4 * bj + ((nd >> 2) & 3), k = 4 * bk + (nd & 3);
    const int g = E.node_off + (lb << 6) + nd;
    const float4 a = acc[g];
    const float m = a.w;
    const bool occ = m > E.eps;
    const v3 mv = f4to3(a);
    const float me = m + E.eps;
    const v3 cur_v = v3{mv.x / me, mv.y / me, mv.z / me};
    const float px = __fmul_rn(__fadd_rn((float)i, 0.5f), E.dx), py = __fmul_rn(__fadd_rn((float)j, 0.5f), E.dx),
                pz = __fmul_rn(__fadd_rn((float)k, 0.5f), E.dx);
    v3 gf = v3{0.f, 0.f, 0.f};
    int4 cid = make_int4(-1, -1, -1, -1);  // argmin per sensor slot (DT_MAX_SENSORS_PER_ENV = 4)
#pragma unroll
    for (int q = 0; q < DT_MAX_SENSORS_PER_ENV; ++q) {
      const int si = E.s_begin + q;
      if (si >= E.s_end) break;
      const int kk = s_cid[it][h][q][nd];
      if (q == 0) cid.x = kk;
      else if (q == 1) cid.y = kk;
      else if (q == 2) cid.z = kk;
      else cid.w = kk;
      if (!occ || kk < 0) continue;
      const dt_sensor& S = w.sensors[si];
      const int4 tr = __ldg(tris + S.f_off + kk);
      SdfRes sr = find_sdf(f4to3(P[tr.x]), f4to3(P[tr.y]), f4to3(P[tr.z]), f4to3(VM[tr.x]), f4to3(VM[tr.y]),
                           f4to3(VM[tr.z]), v3{S.out_dir[0], S.out_dir[1], S.out_dir[2]}, v3{px, py, pz}, cur_v);
      if (!sr.flag) continue;
      const v3 ext = contact_force(E, sr.sdf, sr.n, sr.r);
      gf = gf + w.dt * ext;
      const float4 fe = v3to4(third * (-ext));
      red_add_v4(EXT + tr.x, fe);
      red_add_v4(EXT + tr.y, fe);
      red_add_v4(EXT + tr.z, fe);
    }
    float4 vo = make_float4(0.f, 0.f, 0.f, 0.f);
    if (occ) {
      // grid_op, mpm_elastic.py:220-238
      const float inv_m = 1.f / me;
      v3 u = (inv_m * mv + inv_m * gf) + v3{E.dt_g[0], E.dt_g[1], E.dt_g[2]};
      const int b_ = E.bound;
      if (i < b_ && u.x < 0.f) u.x = 0.f;
      if (i > E.n[0] - b_ && u.x > 0.f) u.x = 0.f;
      if (j < b_ && u.y < 0.f) u.y = 0.f;
      if (j > E.n[1] - b_ && u.y > 0.f) u.y = 0.f;
      if (k < b_ && u.z < 0.f) u.z = 0.f;
      if (k > E.n[2] - b_ && u.z > 0.f) u.z = 0.f;
      if (E.bc == DT_BC_STICKY_FLOOR && j < b_) u = v3{0.f, 0.f, 0.f};
      if (!finite3(u)) set_err(w, DT_DEVERR_NONFINITE);
      vo = v3to4(u);
    }
    vout[g] = vo;
    if (w.skip_tape) {
      // a forward whose tape no backward reads
    } else if (e < w.tape_blocks) {
      const size_t ti = ((size_t)f * w.tape_blocks + e) * 64 + nd;
      reinterpret_cast<float4*>(w.tape_acc)[ti] = a;
      reinterpret_cast<float4*>(w.tape_vout)[ti] = vo;
      reinterpret_cast<int4*>(w.tape_cidx)[ti] = cid;
    } else if (nd == 0) {
      set_err(w, DT_DEVERR_TAPE_FULL);
    }
    acc[g] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (nd == 0) w.blk_flag[b] = 0;
  }
}

// ---------------------------------------------------------------------------------------------
// L3: G2P + FEM integration
// ---------------------------------------------------------------------------------------------
__device__ void g2p_particle(const dt_world& w, int f, int p) {
  const float4 q0 = ldg4(pplane(w, f, 0) + p);
  const v3 x = f4to3(q0);
  const dt_env& E = w.envs[__ldg(w.p_env + p)];
  int base[3];
  float fx[3];
  float* q3n = reinterpret_cast<float*>(pplane(w, f + 1, 3) + p);
  if (!particle_base(E, x, base, fx)) {
    // carry the particle unchanged (its scatter was skipped and the error flag is set)
    pplane(w, f + 1, 0)[p] = q0;
    pplane(w, f + 1, 1)[p] = ldg4(pplane(w, f, 1) + p);
    pplane(w, f + 1, 2)[p] = ldg4(pplane(w, f, 2) + p);
    float4 q3 = ldg4(pplane(w, f, 3) + p);
    *reinterpret_cast<float2*>(q3n) = make_float2(q3.x, q3.y);
    q3n[2] = q3.z;
    return;
  }
  // new v = sum W_o v_o; new C = g2p_k sum W_o v_o (o - fx)^T = g2p_k (S1 - v (fx - 1)^T) with
  // S1 = sum W_o v_o (o - 1)^T, the moment about the stencil's middle node (offsets in {-1, 0, 1}: no
  // cancellation of a large moment against v fx^T): per node one product W v_o and the moment's
  // nonzero columns
  const float4* vout = reinterpret_cast<const float4*>(w.g_vout);
  v3 nv = v3{0.f, 0.f, 0.f};
  m3 S1 = mzero();
  float wts[3][3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int i = 0; i < 3; ++i) wts[i][d] = bsw(i, fx[d]);
#pragma unroll
  for (int oi = 0; oi < 3; ++oi)
#pragma unroll
    for (int oj = 0; oj < 3; ++oj)
#pragma unroll
      for (int ok = 0; ok < 3; ++ok) {
        const v3 gv = f4to3(__ldg(vout + node_index(E, base[0] + oi, base[1] + oj, base[2] + ok)));
        const float W = (wts[oi][0] * wts[oj][1]) * wts[ok][2];
        const v3 Wg = W * gv;
        nv = nv + Wg;
        const float o[3] = {(float)(oi - 1), (float)(oj - 1), (float)(ok - 1)};  // about the middle node
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (o[c] == 0.f) continue;  // resolved at compile time
          S1.a[0][c] += o[c] * Wg.x;
          S1.a[1][c] += o[c] * Wg.y;
          S1.a[2][c] += o[c] * Wg.z;
        }
      }
  m3 nC;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float d = fx[c] - 1.f;
    nC.a[0][c] = E.g2p_k * (S1.a[0][c] - nv.x * d);
    nC.a[1][c] = E.g2p_k * (S1.a[1][c] - nv.y * d);
    nC.a[2][c] = E.g2p_k * (S1.a[2][c] - nv.z * d);
  }
  const v3 nx = x + w.dt * nv;
  if (!finite3(nx)) set_err(w, DT_DEVERR_NONFINITE);
  pplane(w, f + 1, 0)[p] = make_float4(nx.x, nx.y, nx.z, nv.x);
  pplane(w, f + 1, 1)[p] = make_float4(nv.y, nv.z, nC.a[0][0], nC.a[0][1]);
  pplane(w, f + 1, 2)[p] = make_float4(nC.a[0][2], nC.a[1][0], nC.a[1][1], nC.a[1][2]);
  *reinterpret_cast<float2*>(q3n) = make_float2(nC.a[2][0], nC.a[2][1]);
  q3n[2] = nC.a[2][2];
}

__device__ void fem_integrate(const dt_world& w, int f, int i) {
  const dt_sensor& S = w.sensors[__ldg(w.v_sensor + i)];
  const v3 vm = f4to3(vframe(w.v_velmid, w, f)[i]);
  const v3 ex = f4to3(vframe(w.v_ext, w, f)[i]);
  const v3 cvf = f4to3(vframe(w.v_cv, w, f)[i]);
  const v3 cvn = f4to3(vframe(w.v_cv, w, f + 1)[i]);
  v3 vo = vm + S.dt_over_m * ex;
  if (__ldg(w.v_layer + i) == 0) vo = cvf;  // kinematic base layer
  const v3 vel1 = S.carry ? vo + (cvn - cvf) : vo;
  const v3 pos1 = f4to3(vframe(w.v_pos, w, f)[i]) + w.dt * vo;
  const v3 vp1 = f4to3(vframe(w.v_vpos, w, f)[i]) + w.dt * cvf;
  if (!finite3(vel1) || !finite3(pos1)) set_err(w, DT_DEVERR_NONFINITE);
  vframe(w.v_vel, w, f + 1)[i] = v3to4(vel1);
  vframe(w.v_pos, w, f + 1)[i] = v3to4(pos1);
  vframe(w.v_vpos, w, f + 1)[i] = v3to4(vp1);
  // prepare frame f+1's accumulators
  vframe(w.v_velmid, w, f + 1)[i] = v3to4(vel1);
  vframe(w.v_ext, w, f + 1)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

template <int NT, int PPT>
__global__ void __launch_bounds__(NT, DT_MINB(DT_MINB_FWD_G2P, NT)) k_fwd_g2p_fem(dt_world w, int f, int nb_p, int nb_v) {
  pdl_entry();
  int b = blockIdx.x;
  if (b < nb_p) {
    if (PPT == 1) {
      const int p = b * NT + threadIdx.x;
      if (p < w.n_particles) g2p_particle(w, f, p);
    } else {
      int c0, c1;
      cta_chunks(w, NT, PPT, b, c0, c1);
      for (int c = c0; c < c1; ++c) {
        const int p = c * NT + threadIdx.x;
        if (p < w.n_particles) g2p_particle(w, f, p);
      }
    }
    return;
  }
  b -= nb_p;
  if (b < nb_v) {
    int i = b * NT + threadIdx.x;
    if (i < w.n_verts) fem_integrate(w, f, i);
  }
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

inline int check(const dt_world* w, int f) {
  if (!w || f < 0 || f + 1 >= w->n_frames) return DT_ERR_ARG;
  return DT_OK;
}
inline int launched() { return launch_status(cudaGetLastError()); }

template <int MODE, int NT, int PPT>
cudaError_t l1_ppt(const dt_world* w, int f, bool parts, bool fem, cudaStream_t st) {
  const int nb_p = parts ? particle_ctas(w, NT, PPT) : 0;
  const int nb_t = fem ? cdiv(w->n_tets, NT) : 0;
  const int nb_f = fem ? cdiv(w->n_tris, NT) : 0;
  if (nb_p + nb_t + nb_f == 0) return cudaSuccess;
  const size_t smem = scatter_smem(MODE, NT);
  return launch_k(k_fwd_p2g_fem<MODE, NT, PPT>, nb_p + nb_t + nb_f, NT, smem, st, *w, f, nb_p, nb_t, nb_f);
}
template <int MODE, int NT>
cudaError_t l1(const dt_world* w, int f, bool parts, bool fem, cudaStream_t st) {
  return per_thread(w) == 2 ? l1_ppt<MODE, NT, 2>(w, f, parts, fem, st) : l1_ppt<MODE, NT, 1>(w, f, parts, fem, st);
}
template <int MODE>
cudaError_t l1_nt(const dt_world* w, int f, bool parts, bool fem, cudaStream_t st) {
  switch (particle_block(w)) {
    case 64: return l1<MODE, 64>(w, f, parts, fem, st);
    case 256: return l1<MODE, 256>(w, f, parts, fem, st);
    default: return l1<MODE, 128>(w, f, parts, fem, st);
  }
}
int launch_l1(const dt_world* w, int f, bool parts, bool fem, cudaStream_t st) {
  cudaError_t e;
  switch (scatter_kind(w)) {
    case DT_SCATTER_TILE: e = l1<DT_SCATTER_TILE, NT_TILE>(w, f, parts, fem, st); break;
    case DT_SCATTER_GLOBAL: e = l1_nt<DT_SCATTER_GLOBAL>(w, f, parts, fem, st); break;
    case DT_SCATTER_WARP + 1: e = l1_nt<DT_SCATTER_WARP + 1>(w, f, parts, fem, st); break;
    case DT_SCATTER_WARP + 2: e = l1_nt<DT_SCATTER_WARP + 2>(w, f, parts, fem, st); break;
    case DT_MODE_SMEM: e = l1_nt<DT_MODE_SMEM>(w, f, parts, fem, st); break;
    default: e = l1_nt<DT_SCATTER_WARP>(w, f, parts, fem, st);
  }
  return e == cudaSuccess ? DT_OK : DT_ERR_LAUNCH;
}
template <int LPN, bool CAND>
int l2(const dt_world* w, int f, cudaStream_t st) {
  int nb = w->n_blocks < 152 * 8 ? w->n_blocks : 152 * 8;
  if (nb <= 0) return DT_OK;
  const int cap = w->max_sensor_tris < SMEM_CENT_MAX ? w->max_sensor_tris : SMEM_CENT_MAX;
  const size_t smem = stage_bytes(cap);
  static size_t configured[64] = {};
  if (ensure_smem((const void*)k_fwd_grid<LPN, CAND>, smem, configured) != cudaSuccess) return DT_ERR_LAUNCH;
  return launch_status(launch_k(k_fwd_grid<LPN, CAND>, nb, 64 * LPN, smem, st, *w, f, cap));
}
int launch_l2(const dt_world* w, int f, cudaStream_t st) {
  const bool big = w->max_sensor_tris > 32 * DT_CAND_MIN_GROUPS;  // a sensor of more groups than that
  if (w->contact_lanes == 4) return big ? l2<4, true>(w, f, st) : l2<4, false>(w, f, st);
  return big ? l2<8, true>(w, f, st) : l2<8, false>(w, f, st);
}
template <int NT, int PPT>
cudaError_t l3_ppt(const dt_world* w, int f, bool parts, bool fem, cudaStream_t st) {
  const int nb_p = parts ? particle_ctas(w, NT, PPT) : 0;
  const int nb_v = fem ? cdiv(w->n_verts, NT) : 0;
  if (nb_p + nb_v == 0) return cudaSuccess;
  return launch_k(k_fwd_g2p_fem<NT, PPT>, nb_p + nb_v, NT, 0, st, *w, f, nb_p, nb_v);
}
template <int NT>
cudaError_t l3(const dt_world* w, int f, bool parts, bool fem, cudaStream_t st) {
  return per_thread(w) == 2 ? l3_ppt<NT, 2>(w, f, parts, fem, st) : l3_ppt<NT, 1>(w, f, parts, fem, st);
}
int launch_l3(const dt_world* w, int f, bool parts, bool fem, cudaStream_t st) {
  cudaError_t e;
  switch (particle_block(w)) {
    case 64: e = l3<64>(w, f, parts, fem, st); break;
    case 256: e = l3<256>(w, f, parts, fem, st); break;
    default: e = l3<128>(w, f, parts, fem, st);
  }
  return e == cudaSuccess ? DT_OK : DT_ERR_LAUNCH;
}

}  // namespace

extern "C" {

int dt_substep_fwd(const dt_world* w, int f, cudaStream_t stream) {
  int rc = check(w, f);
  if (rc) return rc;
  if ((rc = launch_l1(w, f, true, true, stream))) return rc;
  if ((rc = launch_l2(w, f, stream))) return rc;
  if (w->n_ropes > 0 && has_aux(w)) {
    // the solver reads the rope contact's impulses and writes rope frame f + 1, which nothing in G2P
    // reads: it runs on the aux stream beside G2P and is joined before the call returns
    if ((rc = rope_part(w, f, ROPE_CONTACT, stream))) return rc;
    if (aux_fork(w, stream) != cudaSuccess) return DT_ERR_LAUNCH;
    rc = rope_part(w, f, ROPE_SOLVE, w->aux_stream);
    if (!rc) rc = launch_l3(w, f, true, true, stream);
    // joined on errors too: nothing stays queued on the aux stream past the call
    const cudaError_t j = aux_join(w, stream);
    return rc ? rc : (j == cudaSuccess ? DT_OK : DT_ERR_LAUNCH);
  }
  if ((rc = dt_rope_update(w, f, stream))) return rc;
  return launch_l3(w, f, true, true, stream);
}

int dt_substep_fwd_stage(const dt_world* w, int f, int stage, cudaStream_t stream) {
  int rc = check(w, f);
  if (rc) return rc;
  switch (stage) {
    case 0:
      return launch_l1(w, f, true, true, stream);
    case 1:
      return (rc = launch_l2(w, f, stream)) ? rc : dt_rope_update(w, f, stream);
    case 2:
      return launch_l3(w, f, true, true, stream);
    default:
      return DT_ERR_ARG;
  }
}

int dt_p2g(const dt_world* w, int f, cudaStream_t stream) {
  int rc = check(w, f);
  return rc ? rc : launch_l1(w, f, true, false, stream);
}
int dt_fem_update(const dt_world* w, int f, cudaStream_t stream) {
  int rc = check(w, f);
  return rc ? rc : launch_l1(w, f, false, true, stream);
}
int dt_grid_op(const dt_world* w, int f, cudaStream_t stream) {
  int rc = check(w, f);
  return rc ? rc : launch_l2(w, f, stream);
}
int dt_g2p(const dt_world* w, int f, cudaStream_t stream) {
  int rc = check(w, f);
  return rc ? rc : launch_l3(w, f, true, false, stream);
}
int dt_fem_update2(const dt_world* w, int f, cudaStream_t stream) {
  int rc = check(w, f);
  return rc ? rc : launch_l3(w, f, false, true, stream);
}

}  // extern "C"
