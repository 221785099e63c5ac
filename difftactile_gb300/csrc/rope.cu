// PBD ropes and their contact with the FEM sensors, forward and adjoint.
//
//   rope contact   check_collision + collision, cable_straightening.py:288-319: per rope particle and
//                  env sensor, argmin triangle (contact.cuh), find_sdf with the particle radius as
//                  offset, calculate_contact_force without the clamp of the normal approach speed
//                  (cable_straightening.py:212-224); the rope gets ext * dt (PBD_rope.py:104-105), the
//                  triangle's vertices -ext / 3 (fem_sensor.py:402-406); travel_info set on contact.
//   rope solver    PBDRope.update, PBD_rope.py:112-180: external impulse and gravity, floor (normal
//                  velocity removed, tangential scaled by the friction factor), a Jacobi stretch
//                  pass and a Jacobi bending pass with compliance alpha = c / dt^2 and relaxation
//                  (dt_rope.iters pairs of them; the reference runs one), node 0 pinned, velocity
//                  from the position change.
//
// One CTA per rope holds the rope in shared memory for the solver (a Jacobi pass is a gather of the
// per-constraint corrections, no atomics); the contact search runs four lanes per particle over
// CTAs of 64 particles.  The adjoint recomputes the solver's intermediate positions (in shared memory
// for one pass pair, in the dt_world.r_work workspace for more), runs the passes backwards, applies
// clamp_grid (cable_straightening.py:196-199) and then the contact adjoint with the argmin held from
// the tape.
#include "contact.cuh"

namespace {

constexpr int RC_NT = 256;  // contact: 64 particles x 4 lanes
constexpr int RS_NT = 1024;  // solver: one CTA per rope (about two particles per thread for 2,000)
constexpr int SMEM_CENT_MAX = 12288;  // triangle centroids staged in shared memory (192 KB)
inline int cdiv(int a, int b) { return (a + b - 1) / b; }
inline int launched() { return launch_status(cudaGetLastError()); }

DT_DEV float4* rstate(const dt_world& w, int f, int plane) {
  return reinterpret_cast<float4*>(w.r_state) + ((size_t)f * 2 + plane) * w.n_rope_particles;
}
DT_DEV float4* rext(const dt_world& w, int f) {
  return reinterpret_cast<float4*>(w.r_ext) + (size_t)f * w.n_rope_particles;
}
DT_DEV int4* rcidx(const dt_world& w, int f) {
  return reinterpret_cast<int4*>(w.r_cidx) + (size_t)f * w.n_rope_particles;
}
DT_DEV float4* radj(const dt_world& w, int buf, int plane) {
  return reinterpret_cast<float4*>(w.r_adj) + ((size_t)buf * 2 + plane) * w.n_rope_particles;
}
DT_DEV ContactK rope_k(const dt_rope& R) { return ContactK{R.kn, R.kd, R.kt, R.mu_t, false}; }
DT_DEV float clampr(float a, float c) { return c > 0.f ? fminf(fmaxf(a, -c), c) : a; }

// rope whose contact CTAs contain CTA b
DT_DEV int rope_of_block(const dt_world& w, int b) {
  int r = 0;
  while (r + 1 < w.n_ropes && w.ropes[r + 1].blk_off <= b) ++r;
  return r;
}
// rope holding particle p
DT_DEV int rope_of_particle(const dt_world& w, int p) {
  int r = 0;
  while (r + 1 < w.n_ropes && w.ropes[r + 1].p_off <= p) ++r;
  return r;
}

// ------------------------------------------------------------------------------- forward
// CAND: sensors of more than 32 groups of centroids are searched over per-CTA candidate groups
template <bool CAND>
__global__ void __launch_bounds__(RC_NT) k_rope_contact(dt_world w, int f, int smem_cap) {
  pdl_entry();
  extern __shared__ float4 scent[];
  float4* gbox = scent + smem_cap;
  __shared__ int s_cand[CAND ? SMEM_CENT_MAX / 32 : 1];  // candidate groups of the CTA
  __shared__ int s_box[8];
  const int r = rope_of_block(w, blockIdx.x);
  const dt_rope& R = w.ropes[r];
  const int lp = (blockIdx.x - R.blk_off) * (RC_NT / 4) + (threadIdx.x >> 2), sub = threadIdx.x & 3;
  const bool active = lp < R.n;
  const int p = R.p_off + (active ? lp : 0);
  const float4 s0 = rstate(w, f, 0)[p], s1 = rstate(w, f, 1)[p];
  const v3 x = f4to3(s0), v = f4to3(s1);
  const dt_env& E = w.envs[R.env];
  const ContactK K = rope_k(R);
  const float4* P = vframe(w.v_pos, w, f);
  const float4* VM = vframe(w.v_velmid, w, f);
  float4* EXT = vframe(w.v_ext, w, f);
  const int4* tris = reinterpret_cast<const int4*>(w.tris);
  const float third = 1.f / 3.f;
  v3 es = v3{0.f, 0.f, 0.f};
  bool any = false;
  int4 cid = make_int4(-1, -1, -1, -1);
#pragma unroll
  for (int q = 0; q < DT_MAX_SENSORS_PER_ENV; ++q) {
    const int si = E.s_begin + q;  // block-uniform
    if (si >= E.s_end) break;
    const dt_sensor& S = w.sensors[si];
    const bool in_smem = S.nf <= smem_cap;
    if (in_smem) stage_sensor<RC_NT>(w, S, scent, gbox);
    const int Gall = (S.nf + 31) >> 5;
    int nc = 0;
    const int* cand = nullptr;
    if (CAND && in_smem && Gall > DT_CAND_MIN_GROUPS) {  // block-uniform: the groups any particle of this CTA can need
      if (threadIdx.x == 0) {
        s_box[0] = s_box[1] = s_box[2] = f2ord(3.4e38f);
        s_box[3] = s_box[4] = s_box[5] = f2ord(-3.4e38f);
      }
      __syncthreads();
      const float big = 3.4e38f;
      const float lx = ord_min(active ? x.x : big), ly = ord_min(active ? x.y : big), lz = ord_min(active ? x.z : big);
      const float hx = ord_max(active ? x.x : -big), hy = ord_max(active ? x.y : -big), hz = ord_max(active ? x.z : -big);
      if ((threadIdx.x & 31) == 0) {
        atomicMin(s_box + 0, f2ord(lx));
        atomicMin(s_box + 1, f2ord(ly));
        atomicMin(s_box + 2, f2ord(lz));
        atomicMax(s_box + 3, f2ord(hx));
        atomicMax(s_box + 4, f2ord(hy));
        atomicMax(s_box + 5, f2ord(hz));
      }
      __syncthreads();
      const float4 qlo = make_float4(ord2f(s_box[0]), ord2f(s_box[1]), ord2f(s_box[2]), 0.f);
      const float4 qhi = make_float4(ord2f(s_box[3]), ord2f(s_box[4]), ord2f(s_box[5]), 0.f);
      nc = block_candidates<RC_NT>(gbox, Gall, qlo, qhi, s_cand, s_box + 6);
      cand = s_cand;
    }
    const int kk = closest_tri<4>(w, S, scent, gbox, in_smem, active, x.x, x.y, x.z, sub, cand, nc);
    if (q == 0) cid.x = kk;
    else if (q == 1) cid.y = kk;
    else if (q == 2) cid.z = kk;
    else cid.w = kk;
    if (sub != 0 || !active || kk < 0) continue;
    const int4 tr = __ldg(tris + S.f_off + kk);
    const SdfRes sr = find_sdf(f4to3(P[tr.x]), f4to3(P[tr.y]), f4to3(P[tr.z]), f4to3(VM[tr.x]), f4to3(VM[tr.y]),
                               f4to3(VM[tr.z]), v3{S.out_dir[0], S.out_dir[1], S.out_dir[2]}, x, v, R.rad);
    if (!sr.flag) continue;
    const v3 e = contact_force(K, sr.sdf, sr.n, sr.r);
    es = es + e * w.dt;
    const float4 fe = v3to4(third * (-e));
    red_add_v4(EXT + tr.x, fe);
    red_add_v4(EXT + tr.y, fe);
    red_add_v4(EXT + tr.z, fe);
    any = true;
  }
  if (sub == 0 && active) {
    rext(w, f)[p] = v3to4(es, any ? 1.f : 0.f);
    rcidx(w, f)[p] = cid;
  }
}

// explicit step with external impulse, gravity and floor; .w = 1 where the floor acted
DT_DEV float4 rope_integrate(const dt_rope& R, float dt, float4 s0, float4 s1, float4 e) {
  v3 nv = (f4to3(s1) + f4to3(e) / R.mass) + v3{R.dt_g[0], R.dt_g[1], R.dt_g[2]};
  const float npy = s0.y + nv.y * dt;
  float hit = 0.f;
  if (npy < R.table_h && nv.y < 0.f) {
    nv.y = nv.y - nv.y;
    nv = R.friction * nv;
    hit = 1.f;
  }
  return v3to4(f4to3(s0) + nv * dt, hit);
}

// one Jacobi pass over the constraints (e, e + stride): tp += w * (cd[i] - cd[i - stride])
template <int NTH>
DT_DEV void rope_pass(float4* tp, float4* cd, int n, int stride, float len, float alpha, float relax, float w) {
  for (int e = threadIdx.x; e + stride < n; e += NTH) {
    const v3 d = f4to3(tp[e]) - f4to3(tp[e + stride]);
    const float L = sqrtf(dot(d, d) + 1e-10f);
    const float k = -(L - len) / (w + w + alpha);
    cd[e] = make_float4(k * d.x / L * relax, k * d.y / L * relax, k * d.z / L * relax, 0.f);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += NTH) {
    v3 acc = v3{0.f, 0.f, 0.f};
    if (i - stride >= 0) acc = acc - f4to3(cd[i - stride]) * w;
    if (i + stride < n) acc = acc + f4to3(cd[i]) * w;
    const float4 t = tp[i];
    tp[i] = v3to4(f4to3(t) + acc, t.w);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(RS_NT) k_rope_solve(dt_world w, int f) {
  pdl_entry();
  extern __shared__ float4 sm[];
  const dt_rope& R = w.ropes[blockIdx.x];
  const int n = R.n;
  float4* tp = sm;
  float4* cd = sm + w.max_rope_n;
  const float dt = w.dt;
  for (int i = threadIdx.x; i < n; i += RS_NT) {
    const int p = R.p_off + i;
    tp[i] = rope_integrate(R, dt, rstate(w, f, 0)[p], rstate(w, f, 1)[p], rext(w, f)[p]);
  }
  __syncthreads();
  const int iters = R.iters > 1 ? R.iters : 1;
  for (int it = 0; it < iters; ++it) {
    rope_pass<RS_NT>(tp, cd, n, 1, R.rest, R.alpha_s, R.relax_s, R.inv_m);
    rope_pass<RS_NT>(tp, cd, n, 2, R.bend, R.alpha_b, R.relax_b, R.inv_m);
  }
  for (int i = threadIdx.x; i < n; i += RS_NT) {
    const int p = R.p_off + i;
    const float4 s0 = rstate(w, f, 0)[p];
    const v3 x1 = i == 0 ? v3{R.pin[0], R.pin[1], R.pin[2]} : f4to3(tp[i]);
    const v3 v1 = (x1 - f4to3(s0)) / dt;
    if (!finite3(x1) || !finite3(v1)) set_err(w, DT_DEVERR_NONFINITE);
    const float trav = rext(w, f)[p].w != 0.f ? 1.f : s0.w;
    rstate(w, f + 1, 0)[p] = v3to4(x1, trav);
    rstate(w, f + 1, 1)[p] = v3to4(v1, 0.f);
  }
}

// ------------------------------------------------------------------------------- adjoint
// adjoint of one Jacobi pass at input positions tp: tpb (d/d output on entry) += J^T tpb
template <int NTH>
DT_DEV void rope_pass_bwd(const float4* tp, float4* tpb, float4* cd, int n, int stride, float len, float alpha,
                          float relax, float w) {
  const float k = -relax / (w + w + alpha);
  for (int e = threadIdx.x; e + stride < n; e += NTH) {
    const v3 d = f4to3(tp[e]) - f4to3(tp[e + stride]);
    const float L = sqrtf(dot(d, d) + 1e-10f);
    const v3 dpb = w * (f4to3(tpb[e]) - f4to3(tpb[e + stride]));
    const float a = k * (L - len) / L;
    const float bco = k * len / (L * L * L) * dot(d, dpb);
    cd[e] = v3to4(a * dpb + bco * d);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += NTH) {
    v3 add = v3{0.f, 0.f, 0.f};
    if (i - stride >= 0) add = add - f4to3(cd[i - stride]);
    if (i + stride < n) add = add + f4to3(cd[i]);
    tpb[i] = v3to4(f4to3(tpb[i]) + add);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(RS_NT) k_rope_solve_bwd(dt_world w, int f) {
  pdl_entry();
  extern __shared__ float4 sm[];
  const dt_rope& R = w.ropes[blockIdx.x];
  const int n = R.n, M = w.max_rope_n;
  float4* tp0 = sm;
  float4* tp1 = sm + M;
  float4* tpb = sm + 2 * M;
  float4* cd = sm + 3 * M;
  const float dt = w.dt;
  const int b1 = (f + 1) & 1, b0 = f & 1;
  const int iters = R.iters > 1 ? R.iters : 1;
  if (iters > 1 && (w.r_work == nullptr || iters > w.max_rope_iters)) {  // no room for the pass inputs
    if (threadIdx.x == 0) set_err(w, DT_DEVERR_ROPE_ITERS);
    return;
  }
  for (int i = threadIdx.x; i < n; i += RS_NT) {
    const int p = R.p_off + i;
    const float4 t = rope_integrate(R, dt, rstate(w, f, 0)[p], rstate(w, f, 1)[p], rext(w, f)[p]);
    tp0[i] = t;
    tp1[i] = t;
    // vel1 = (pos1 - pos) / dt, pos1[0] = pin, pos1[i] = tp2[i]
    const v3 pb1 = f4to3(radj(w, b1, 0)[p]), vb1 = f4to3(radj(w, b1, 1)[p]);
    tpb[i] = i == 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : v3to4(pb1 + vb1 / dt);
  }
  __syncthreads();
  if (iters == 1) {  // the pass inputs fit in shared memory: tp0 (stretch), tp1 (bending)
    rope_pass<RS_NT>(tp1, cd, n, 1, R.rest, R.alpha_s, R.relax_s, R.inv_m);
    rope_pass_bwd<RS_NT>(tp1, tpb, cd, n, 2, R.bend, R.alpha_b, R.relax_b, R.inv_m);
    rope_pass_bwd<RS_NT>(tp0, tpb, cd, n, 1, R.rest, R.alpha_s, R.relax_s, R.inv_m);
  } else {
    // every pass's input positions into the workspace (pass k of this rope at r_work[k][p_off ..]),
    // then the passes backwards
    const size_t NR = (size_t)w.n_rope_particles;
    float4* work = reinterpret_cast<float4*>(w.r_work) + R.p_off;
    for (int k = 0; k < 2 * iters; ++k) {
      for (int i = threadIdx.x; i < n; i += RS_NT) work[k * NR + i] = tp1[i];
      // each pass ends with __syncthreads(), which also orders these writes before the backward
      // passes read them from other threads of the CTA
      if (k & 1) rope_pass<RS_NT>(tp1, cd, n, 2, R.bend, R.alpha_b, R.relax_b, R.inv_m);
      else rope_pass<RS_NT>(tp1, cd, n, 1, R.rest, R.alpha_s, R.relax_s, R.inv_m);
    }
    for (int it = iters - 1; it >= 0; --it) {
      rope_pass_bwd<RS_NT>(work + (2 * it + 1) * NR, tpb, cd, n, 2, R.bend, R.alpha_b, R.relax_b, R.inv_m);
      rope_pass_bwd<RS_NT>(work + (2 * it) * NR, tpb, cd, n, 1, R.rest, R.alpha_s, R.relax_s, R.inv_m);
    }
  }
  const float clip = w.grad_clip;
  for (int i = threadIdx.x; i < n; i += RS_NT) {
    const int p = R.p_off + i;
    const float4 a1 = radj(w, b1, 0)[p];
    const v3 vb1 = f4to3(radj(w, b1, 1)[p]);
    const v3 tb = f4to3(tpb[i]);
    v3 xb = (-1.f * vb1) / dt + tb;
    v3 nvb = tb * dt;
    if (tp0[i].w != 0.f) nvb = v3{R.friction * nvb.x, 0.f, R.friction * nvb.z};
    const v3 reb = nvb / R.mass;
    xb = v3{clampr(xb.x, clip), clampr(xb.y, clip), clampr(xb.z, clip)};
    nvb = v3{clampr(nvb.x, clip), clampr(nvb.y, clip), clampr(nvb.z, clip)};
    const float travb = rext(w, f)[p].w != 0.f ? 0.f : a1.w;
    radj(w, b0, 0)[p] = v3to4(xb, travb);
    radj(w, b0, 1)[p] = v3to4(nvb, 0.f);
    reinterpret_cast<float4*>(w.r_extb)[p] = v3to4(reb);
  }
}

// contact adjoint per rope particle (argmin from the tape); one thread per particle
__global__ void __launch_bounds__(128) k_rope_contact_bwd(dt_world w, int f) {
  pdl_entry();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= w.n_rope_particles) return;
  const float4 e = rext(w, f)[p];
  if (e.w == 0.f) return;
  const dt_rope& R = w.ropes[rope_of_particle(w, p)];
  const dt_env& E = w.envs[R.env];
  const ContactK K = rope_k(R);
  const int4 c4 = rcidx(w, f)[p];
  const int cid[4] = {c4.x, c4.y, c4.z, c4.w};
  const v3 x = f4to3(rstate(w, f, 0)[p]), v = f4to3(rstate(w, f, 1)[p]);
  const v3 reb = f4to3(reinterpret_cast<const float4*>(w.r_extb)[p]);
  const size_t V = (size_t)w.n_verts;
  const float4* P = vframe(w.v_pos, w, f);
  const float4* VM = vframe(w.v_velmid, w, f);
  float4* aPos = reinterpret_cast<float4*>(w.v_adj_pos) + (size_t)(f & 1) * V;
  float4* aVm = reinterpret_cast<float4*>(w.v_adj_velmid);
  const float4* aExt = reinterpret_cast<const float4*>(w.v_adj_ext);
  const int4* tris = reinterpret_cast<const int4*>(w.tris);
  const float third = 1.f / 3.f;
  v3 xb = v3{0.f, 0.f, 0.f}, vb = v3{0.f, 0.f, 0.f};
  for (int q = 0; q < DT_MAX_SENSORS_PER_ENV; ++q) {
    const int si = E.s_begin + q;
    if (si >= E.s_end) break;
    if (cid[q] < 0) continue;
    const dt_sensor& S = w.sensors[si];
    const int4 tr = __ldg(tris + S.f_off + cid[q]);
    const v3 p1 = f4to3(P[tr.x]), p2 = f4to3(P[tr.y]), p3 = f4to3(P[tr.z]);
    const v3 od = v3{S.out_dir[0], S.out_dir[1], S.out_dir[2]};
    const SdfRes sr = find_sdf(p1, p2, p3, f4to3(VM[tr.x]), f4to3(VM[tr.y]), f4to3(VM[tr.z]), od, x, v, R.rad);
    if (!sr.flag) continue;
    const v3 exs = (f4to3(aExt[tr.x]) + f4to3(aExt[tr.y])) + f4to3(aExt[tr.z]);
    const v3 eb = w.dt * reb - third * exs;
    v3 nb = v3{0.f, 0.f, 0.f}, rb = v3{0.f, 0.f, 0.f};
    const float sdfb = contact_force_bwd(K, sr.sdf, sr.n, sr.r, eb, nb, rb);
    const v3 tvb = third * rb;
    red_add_v4(aVm + tr.x, v3to4(tvb));
    red_add_v4(aVm + tr.y, v3to4(tvb));
    red_add_v4(aVm + tr.z, v3to4(tvb));
    vb = vb - rb;
    xb = xb + sdfb * sr.n;
    v3 b1, b2, b3;
    tri_geom_bwd(p1, p2, p3, od, x, sr.n, sdfb, nb, b1, b2, b3);
    red_add_v4(aPos + tr.x, v3to4(b1));
    red_add_v4(aPos + tr.y, v3to4(b2));
    red_add_v4(aPos + tr.z, v3to4(b3));
  }
  float4* ax = radj(w, f & 1, 0) + p;
  float4* av = radj(w, f & 1, 1) + p;
  const float4 a = *ax, b = *av;
  *ax = make_float4(a.x + xb.x, a.y + xb.y, a.z + xb.z, a.w);
  *av = make_float4(b.x + vb.x, b.y + vb.y, b.z + vb.z, b.w);
}

int set_smem(const void* fn, size_t bytes, size_t (&configured)[64]) {
  return ensure_smem(fn, bytes, configured) == cudaSuccess ? DT_OK : DT_ERR_CAPACITY;
}


}  // namespace

// the parts of dt_rope_update / dt_rope_update_bwd, for the substep drivers that overlap the solver
// with the MPM stages (declared in common.cuh)
int rope_part(const dt_world* w, int f, int part, cudaStream_t stream) {
  if (w->n_ropes <= 0) return DT_OK;
  int rc;
  if (part == ROPE_CONTACT || part == ROPE_SOLVE) {
    if (!w->ropes || !w->r_state || !w->r_ext || !w->r_cidx || w->max_rope_n <= 0) return DT_ERR_ARG;
    const size_t solve_smem = (size_t)2 * w->max_rope_n * sizeof(float4);
    if (solve_smem > 227 * 1024) return DT_ERR_CAPACITY;
    if (part == ROPE_SOLVE) {
      static size_t conf_s[64] = {};
      if ((rc = set_smem((const void*)k_rope_solve, solve_smem, conf_s))) return rc;
      return launch_k(k_rope_solve, w->n_ropes, RS_NT, solve_smem, stream, *w, f) == cudaSuccess ? DT_OK
                                                                                                  : DT_ERR_LAUNCH;
    }
    const int cap = w->max_sensor_tris < SMEM_CENT_MAX ? w->max_sensor_tris : SMEM_CENT_MAX;
    const size_t smem = stage_bytes(cap);
    static size_t conf_c[64] = {}, conf_cc[64] = {};
    const bool big = w->max_sensor_tris > 32 * DT_CAND_MIN_GROUPS;  // a sensor of more groups than that
    if ((rc = set_smem(big ? (const void*)k_rope_contact<true> : (const void*)k_rope_contact<false>, smem,
                       big ? conf_cc : conf_c)))
      return rc;
    if (w->rope_blocks > 0 &&
        launch_k(big ? k_rope_contact<true> : k_rope_contact<false>, w->rope_blocks, RC_NT, smem, stream, *w, f,
                 cap) != cudaSuccess)
      return DT_ERR_LAUNCH;
    return DT_OK;
  }
  if (!w->ropes || !w->r_adj || !w->r_extb || w->max_rope_n <= 0) return DT_ERR_ARG;
  if (part == ROPE_SOLVE_BWD) {
    const size_t smem = (size_t)4 * w->max_rope_n * sizeof(float4);
    if (smem > 227 * 1024) return DT_ERR_CAPACITY;
    static size_t conf[64] = {};
    if ((rc = set_smem((const void*)k_rope_solve_bwd, smem, conf))) return rc;
    return launch_k(k_rope_solve_bwd, w->n_ropes, RS_NT, smem, stream, *w, f) == cudaSuccess ? DT_OK : DT_ERR_LAUNCH;
  }
  if (part == ROPE_CONTACT_BWD)
    return launch_k(k_rope_contact_bwd, cdiv(w->n_rope_particles, 128), 128, 0, stream, *w, f) == cudaSuccess
               ? DT_OK
               : DT_ERR_LAUNCH;
  return DT_ERR_ARG;
}

extern "C" {

int dt_rope_update(const dt_world* w, int f, cudaStream_t stream) {
  if (!w || f < 0 || f + 1 >= w->n_frames) return DT_ERR_ARG;
  int rc = rope_part(w, f, ROPE_CONTACT, stream);
  return rc ? rc : rope_part(w, f, ROPE_SOLVE, stream);
}

int dt_rope_update_bwd(const dt_world* w, int f, cudaStream_t stream) {
  if (!w || f < 0 || f + 1 >= w->n_frames) return DT_ERR_ARG;
  int rc = rope_part(w, f, ROPE_SOLVE_BWD, stream);
  return rc ? rc : rope_part(w, f, ROPE_CONTACT_BWD, stream);
}

}  // extern "C"
