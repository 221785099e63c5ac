// Adjoint substep kernels (sm_103a): the reverse of Contact.update (grasp_plastic.py:151-164)
// in the order of Contact.update_grad (grasp_plastic.py:167-178):
//   B0 k_bwd_restore   : grid velocities of frame f back from the tape into the dense grid
//   B1 k_bwd_g2p_fem   : particles — G2P adjoint (scatter into the grid adjoint, x adjoint);
//                        vertices  — FEM integration adjoint + clamp_grid on sensor grads
//   B2 k_bwd_grid      : active blocks of frame f — grid_op adjoint, clamp of the grid-mass grad,
//                        contact adjoint (argmin held constant, as the reference computes it in a
//                        non-differentiated kernel) into grid and sensor adjoints
//   B3 k_bwd_p2g_fem   : particles — P2G adjoint (gather), stress/return-map adjoint, SVD adjoint
//                        of mpm_elastic.py:145-173 (1/(s_j^2-s_i^2) clamped at +-1e-8),
//                        F-update adjoint, material (mu, lambda) grads;
//                        tets      — FEM elastic-force adjoint into position grads;
//                        vertices  — velocity adjoint of frame f
// Adjoint of frame f+1 is read from buffer (f+1)&1, adjoint of frame f written to buffer f&1.
#include "common.cuh"

namespace {

constexpr int NT_TILE = 128;  // threads per CTA of the G2P adjoint with the TILE scatter
constexpr int GRID_NT = 64;
constexpr int TILE_MAX = 1728;  // shared scatter tile capacity in nodes (12^3)

DT_DEV float clampg(float a, float c) { return c > 0.f ? fminf(fmaxf(a, -c), c) : a; }
DT_DEV v3 clampg(v3 a, float c) { return v3{clampg(a.x, c), clampg(a.y, c), clampg(a.z, c)}; }
DT_DEV float4 ld4(const float4* p) { return *p; }

// c (y^p - x^p) / (y - x) for x, y > 0 from the values fx = c x^p, fy = c y^p and gx = c x^(p-1):
// the quotient itself, or where x and y are within 1% (the quotient would cancel) its series in
// t = (y - x) / x, p gx (1 + q t / 2 + q (q-1) t^2 / 6 + q (q-1) (q-2) t^3 / 24) with q = p - 1
DT_DEV float cdd(float x, float y, float fx, float fy, float gx, float p) {
  const float h = y - x;
  if (fabsf(h) > 1e-2f * fmaxf(x, y)) return (fy - fx) / h;
  const float t = h / x, q = p - 1.f;
  return p * gx * (1.f + t * (0.5f * q + t * (q * (q - 1.f) / 6.f + t * (q * (q - 1.f) * (q - 2.f) / 24.f))));
}

// the reference's clamp of the singular-value gap (mpm_elastic.py:150-155)
DT_DEV float gap_clamp(float a) { return a >= 0.f ? fmaxf(a, 1e-8f) : fminf(a, -1e-8f); }

// SVD adjoint, mpm_elastic.py:158-173: F_bar = U [ (ff o (U^T Ub - Ub^T U)) S + diag(sb)
// + S (ff o (V^T Vb - Vb^T V)) ] V^T with ff_ij = 1/clamp(s_j^2 - s_i^2).  The adjoint Rb of the
// rotation R = U V^T is passed separately: with M = U^T Rb V it contributes Ub = Rb V, Vb = Rb^T U,
// i.e. ff_ij (M - M^T)_ij (s_j - s_i), which the stable mode evaluates as (M - M^T)_ij / (s_i + s_j).
// uv false: the caller's Ub and Vb are zero, and in the stable mode their ff terms (zero) are skipped
// (the result differs at most in the sign of an exact zero).  `extra` is added to the bracket before
// the final U [.] V^T (a caller's own term of that form, for one product instead of two).
DT_DEV m3 svd_grad(const m3& U, v3 s, const m3& V, const m3& Ub_in, v3 sb, const m3& Vb_in, const m3& Rb, int mode,
                   bool uv = true, const m3& extra = mzero()) {
  const float sv[3] = {s.x, s.y, s.z};
  m3 Ub = Ub_in, Vb = Vb_in;
  if (mode == DT_SVDGRAD_REFERENCE) {
    Ub = madd(Ub, mmul(Rb, V));
    Vb = madd(Vb, mTmul(Rb, U));
    uv = true;
  }
  const m3 M = mmul(mTmul(U, Rb), V);
  m3 inner;
  if (uv) {
    const m3 UtUb = mTmul(U, Ub), UbtU = mTmul(Ub, U), VtVb = mTmul(V, Vb), VbtV = mTmul(Vb, V);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        float v = 0.f;
        if (i != j) {
          const float ff = 1.f / gap_clamp(sv[j] * sv[j] - sv[i] * sv[i]);
          v = ff * (UtUb.a[i][j] - UbtU.a[i][j]) * sv[j] + sv[i] * ff * (VtVb.a[i][j] - VbtV.a[i][j]);
          if (mode != DT_SVDGRAD_REFERENCE) v += (M.a[i][j] - M.a[j][i]) / gap_clamp(sv[i] + sv[j]);
        } else {
          v = i == 0 ? sb.x : (i == 1 ? sb.y : sb.z);
        }
        inner.a[i][j] = v;
      }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        inner.a[i][j] = i != j ? (M.a[i][j] - M.a[j][i]) / gap_clamp(sv[i] + sv[j])
                               : (i == 0 ? sb.x : (i == 1 ? sb.y : sb.z));
  }
  return mmulT(mmul(U, madd(inner, extra)), V);
}

// ---------------------------------------------------------------------------------------------
// B0
// ---------------------------------------------------------------------------------------------
// grid velocities of frame f back from the tape: `per` blocks per CTA pass (64 threads each)
DT_DEV void restore_blocks(const dt_world& w, int f, int cta, int ncta, int per) {
  const int cnt = min(w.tape_bcount[f], w.tape_blocks);
  const int l = threadIdx.x & 63;
  for (int e = cta * per + (threadIdx.x >> 6); e < cnt; e += ncta * per) {
    const int b = w.tape_blist[(size_t)f * w.n_blocks + e];
    const dt_env& E = w.envs[__ldg(w.blk_env + b)];
    const int g = E.node_off + ((b - E.blk_off) << 6) + l;
    reinterpret_cast<float4*>(w.g_vout)[g] =
        reinterpret_cast<const float4*>(w.tape_vout)[((size_t)f * w.tape_blocks + e) * 64 + l];
  }
}

__global__ void __launch_bounds__(GRID_NT) k_bwd_restore(dt_world w, int f) {
  pdl_entry();
  restore_blocks(w, f, blockIdx.x, gridDim.x, 1);
}

// ---------------------------------------------------------------------------------------------
// B1
// ---------------------------------------------------------------------------------------------
// G2P adjoint of one CTA's particles: the position adjoint needs the grid velocities (a gather);
// the grid-velocity adjoint W (vn_bar + 4 inv_dx C_bar (o - fx)) = W (q + o . c) is a 27-node
// scatter, privatised through the shared-memory tile.
template <int MODE, int NT>
__device__ void g2p_bwd_chunk(const dt_world& w, int f, int chunk, float4* tile, int* sh) {
  const int p = chunk * NT + threadIdx.x;
  const bool valid = p < w.n_particles;
  const int nb = (f + 1) & 1, cb = f & 1;
  int base[3] = {0, 0, 0};
  float fx[3] = {0.f, 0.f, 0.f};
  bool ok = false;
  int env = 0;
  float wx[3] = {0.f, 0.f, 0.f}, wy[3] = {0.f, 0.f, 0.f}, wz[3] = {0.f, 0.f, 0.f};
  v3 q = v3{0.f, 0.f, 0.f}, c0 = q, c1 = q, c2 = q;
  if (valid) {
    const float4 a0 = ld4(padj(w, nb, 0) + p), a1 = ld4(padj(w, nb, 1) + p), a2 = ld4(padj(w, nb, 2) + p),
                 a3 = ld4(padj(w, nb, 3) + p);
    const v3 xb1 = v3{a0.x, a0.y, a0.z};
    const v3 vb1 = v3{a0.w, a1.x, a1.y};
    m3 Cb;
    Cb.a[0][0] = a1.z;
    Cb.a[0][1] = a1.w;
    Cb.a[0][2] = a2.x;
    Cb.a[1][0] = a2.y;
    Cb.a[1][1] = a2.z;
    Cb.a[1][2] = a2.w;
    Cb.a[2][0] = a3.x;
    Cb.a[2][1] = a3.y;
    Cb.a[2][2] = a3.z;
    const v3 x = f4to3(ldg4(pplane(w, f, 0) + p));
    env = __ldg(w.p_env + p);
    const dt_env& E = w.envs[env];
    float4* out0 = padj(w, cb, 0) + p;
    ok = particle_base(E, x, base, fx);
    if (!ok) {
      *out0 = make_float4(xb1.x, xb1.y, xb1.z, 0.f);  // carried unchanged in the forward pass
    } else {
      const v3 vnb = vb1 + w.dt * xb1;  // x_new = x + dt v_new
      float fxb[3] = {0.f, 0.f, 0.f};
      const float4* vout = reinterpret_cast<const float4*>(w.g_vout);
      float dws[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        wx[i] = bsw(i, fx[0]);
        wy[i] = bsw(i, fx[1]);
        wz[i] = bsw(i, fx[2]);
        dws[i][0] = bsdw(i, fx[0]);
        dws[i][1] = bsdw(i, fx[1]);
        dws[i][2] = bsdw(i, fx[2]);
      }
      // With v_o the grid velocity of node o:  Wb_o = v_o . (vnb + g2p_k C_bar (o - fx)) = v_o . u_o,
      // u_o = u_1 + sum_c (o_c - 1) k_c  (u_1 = vnb + g2p_k C_bar (1 - fx), the middle node's;
      // k_c = g2p_k C_bar column c), and the weight-independent part of fx_bar,
      // -g2p_k sum_o W_o C_bar^T v_o, is -g2p_k C_bar^T S0 with S0 = sum W_o v_o, applied after the loop
      const float gk = E.g2p_k;
      const v3 k0 = gk * mcol(Cb, 0), k1 = gk * mcol(Cb, 1), k2 = gk * mcol(Cb, 2);
      const v3 u1 = vnb + mvec(Cb, v3{(1.f - fx[0]) * gk, (1.f - fx[1]) * gk, (1.f - fx[2]) * gk});
      v3 S0 = v3{0.f, 0.f, 0.f};
      const StencilNodes sn = stencil_nodes(E, base);
#pragma unroll
      for (int oi = 0; oi < 3; ++oi) {
        const v3 ui = oi == 0 ? u1 - k0 : (oi == 1 ? u1 : u1 + k0);  // offsets about the middle node
#pragma unroll
        for (int oj = 0; oj < 3; ++oj) {
          const v3 uij = oj == 0 ? ui - k1 : (oj == 1 ? ui : ui + k1);
          float Z = 0.f, Zd = 0.f;  // the row's sum_k wz_k Wb and sum_k dwz_k Wb
#pragma unroll
          for (int ok_ = 0; ok_ < 3; ++ok_) {
            const v3 u = ok_ == 0 ? uij - k2 : (ok_ == 1 ? uij : uij + k2);
            const v3 gv = f4to3(__ldg(vout + ((sn.x[oi] + sn.y[oj]) + sn.z[ok_])));
            const float W = (wx[oi] * wy[oj]) * wz[ok_];
            const float Wb = dot(gv, u);
            S0 = S0 + W * gv;
            Z += wz[ok_] * Wb;
            Zd += dws[ok_][2] * Wb;
          }
          fxb[0] += (dws[oi][0] * wy[oj]) * Z;
          fxb[1] += (wx[oi] * dws[oj][1]) * Z;
          fxb[2] += (wx[oi] * wy[oj]) * Zd;
        }
      }
      const v3 CtS0 = mTvec(Cb, S0);
      fxb[0] -= gk * CtS0.x;
      fxb[1] -= gk * CtS0.y;
      fxb[2] -= gk * CtS0.z;
      const v3 xb = xb1 + E.inv_dx * v3{fxb[0], fxb[1], fxb[2]};
      *out0 = make_float4(xb.x, xb.y, xb.z, 0.f);
      c0 = k0;
      c1 = k1;
      c2 = k2;
      q = u1;
    }
  }
  StencilRec rec;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    rec.wx[i] = wx[i];
    rec.wy[i] = wy[i];
    rec.wz[i] = wz[i];
  }
  rec.q = make_float4(q.x, q.y, q.z, 0.f);
  rec.c0 = c0;
  rec.c1 = c1;
  rec.c2 = c2;
  auto no_box = [](const dt_env&, int, int, int, int, int, int, int, int) {};
  auto no_one = [](const dt_env&) {};
  stencil_scatter<NT, TILE_MAX, MODE, false>(w, chunk, ok, env, base, rec, reinterpret_cast<float*>(tile), sh,
                                reinterpret_cast<float4*>(w.g_adj_vout), no_box, no_one);
}

__device__ void integrate_bwd(const dt_world& w, int f, int i) {
  const int nb = (f + 1) & 1, cb = f & 1;
  const dt_sensor& S = w.sensors[__ldg(w.v_sensor + i)];
  const size_t V = (size_t)w.n_verts;
  const v3 posb1 = f4to3(reinterpret_cast<const float4*>(w.v_adj_pos)[nb * V + i]);
  const v3 velb1 = f4to3(reinterpret_cast<const float4*>(w.v_adj_vel)[nb * V + i]);
  const v3 vpb1 = f4to3(reinterpret_cast<const float4*>(w.v_adj_vpos)[nb * V + i]);
  float4* cvb_f = vframe(w.v_adj_cv, w, f) + i;
  float4* cvb_n = vframe(w.v_adj_cv, w, f + 1) + i;
  v3 cvb = f4to3(*cvb_f);
  v3 cvbn = f4to3(*cvb_n);
  // vpos1 = vpos + dt cv ; pos1 = pos + dt vo ; vel1 = vo + carry (cv1 - cv)
  cvb = cvb + w.dt * vpb1;
  v3 vob = velb1 + w.dt * posb1;
  if (S.carry) {
    cvbn = cvbn + velb1;
    cvb = cvb - velb1;
  }
  v3 vmb = v3{0.f, 0.f, 0.f}, exb = v3{0.f, 0.f, 0.f};
  if (__ldg(w.v_layer + i) == 0) {
    cvb = cvb + vob;
  } else {
    vmb = vob;
    exb = S.dt_over_m * vob;
  }
  // clamp_grid on the sensor's pos/vel grads of frame f (grasp_plastic.py:196-202)
  const v3 posb = clampg(posb1, w.grad_clip);
  vmb = clampg(vmb, w.grad_clip);
  reinterpret_cast<float4*>(w.v_adj_pos)[cb * V + i] = v3to4(posb);
  reinterpret_cast<float4*>(w.v_adj_vpos)[cb * V + i] = v3to4(vpb1);
  reinterpret_cast<float4*>(w.v_adj_velmid)[i] = v3to4(vmb);
  // v_adj_ext accumulates: a readout of frame f's contact forces may have seeded it (it is reset
  // after its last use in stage 3)
  float4* ae = reinterpret_cast<float4*>(w.v_adj_ext) + i;
  const float4 ae0 = *ae;
  *ae = make_float4(ae0.x + exb.x, ae0.y + exb.y, ae0.z + exb.z, 0.f);
  *cvb_f = v3to4(cvb);
  if (S.carry) *cvb_n = v3to4(cvbn);
}

template <int MODE, int NT, int PPT>
__global__ void __launch_bounds__(NT, DT_MINB(DT_MINB_BWD_G2P, NT)) k_bwd_g2p_fem(dt_world w, int f, int nb_p, int nb_v) {
  pdl_entry();
  extern __shared__ float4 tile[];  // stencil records (TILE mode) or the grid tile (SMEM mode); none otherwise
  __shared__ int sh[8];
  int b = blockIdx.x;
  if (b < nb_p) {
    if (PPT == 1) {
      g2p_bwd_chunk<MODE, NT>(w, f, b, tile, sh);
    } else {
      int c0, c1;
      cta_chunks(w, NT, PPT, b, c0, c1);
      for (int c = c0; c < c1; ++c) {
        // the shared tile of the previous chunk (the modes without one share nothing between chunks)
        if (c > c0 && (MODE == DT_SCATTER_TILE || MODE >= DT_MODE_SMEM)) __syncthreads();
        g2p_bwd_chunk<MODE, NT>(w, f, c, tile, sh);
      }
    }
    return;
  }
  b -= nb_p;
  if (b < nb_v) {
    int i = b * NT + threadIdx.x;
    if (i < w.n_verts) integrate_bwd(w, f, i);
  }
}

// ---------------------------------------------------------------------------------------------
// B2: grid op + contact adjoint
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(GRID_NT, DT_MINB(DT_MINB_BWD_GRID, GRID_NT)) k_bwd_grid(dt_world w, int f) {
  pdl_entry();
  const int cnt = min(w.tape_bcount[f], w.tape_blocks);
  const int l = threadIdx.x;
  const float third = 1.f / 3.f;
  const int cb = f & 1;
  const size_t V = (size_t)w.n_verts;
  float4* avout = reinterpret_cast<float4*>(w.g_adj_vout);
  float4* aacc = reinterpret_cast<float4*>(w.g_adj_acc);
  const float4* P = vframe(w.v_pos, w, f);
  const float4* VM = vframe(w.v_velmid, w, f);
  float4* aPos = reinterpret_cast<float4*>(w.v_adj_pos) + cb * V;
  float4* aVm = reinterpret_cast<float4*>(w.v_adj_velmid);
  const float4* aExt = reinterpret_cast<const float4*>(w.v_adj_ext);
  const int4* tris = reinterpret_cast<const int4*>(w.tris);
  for (int e = blockIdx.x; e < cnt; e += gridDim.x) {
    const int b = w.tape_blist[(size_t)f * w.n_blocks + e];
    const dt_env& E = w.envs[__ldg(w.blk_env + b)];
    const int lb = b - E.blk_off;
    const int bk = lb % E.nb[2], bj = (lb / E.nb[2]) % E.nb[1], bi = lb / (E.nb[1] * E.nb[2]);
    const int i = 4 * bi + (l >> 4), j = 4 * bj + ((l >> 2) & 3), k = 4 * bk + (l & 3);
    const int g = E.node_off + (lb << 6) + l;
    const size_t ti = ((size_t)f * w.tape_blocks + e) * 64 + l;
    const float4 a = reinterpret_cast<const float4*>(w.tape_acc)[ti];
    const int4 cid4 = reinterpret_cast<const int4*>(w.tape_cidx)[ti];
    const v3 vb = f4to3(avout[g]);
    avout[g] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float m = a.w;
    float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
    if (m > E.eps) {
      const v3 mv = f4to3(a);
      const float me = m + E.eps;
      const float inv_m = 1.f / me;
      const v3 cur_v = v3{mv.x / me, mv.y / me, mv.z / me};
      const v3 p = v3{__fmul_rn(__fadd_rn((float)i, 0.5f), E.dx), __fmul_rn(__fadd_rn((float)j, 0.5f), E.dx),
                      __fmul_rn(__fadd_rn((float)k, 0.5f), E.dx)};
      const int cid[4] = {cid4.x, cid4.y, cid4.z, cid4.w};
      // forward recompute of the contact force sum
      v3 gf = v3{0.f, 0.f, 0.f};
#pragma unroll
      for (int q = 0; q < DT_MAX_SENSORS_PER_ENV; ++q) {
        const int si = E.s_begin + q;
        if (si >= E.s_end) break;
        if (cid[q] < 0) continue;
        const dt_sensor& S = w.sensors[si];
        const int4 tr = __ldg(tris + S.f_off + cid[q]);
        SdfRes sr = find_sdf(f4to3(P[tr.x]), f4to3(P[tr.y]), f4to3(P[tr.z]), f4to3(VM[tr.x]), f4to3(VM[tr.y]),
                             f4to3(VM[tr.z]), v3{S.out_dir[0], S.out_dir[1], S.out_dir[2]}, p, cur_v);
        if (!sr.flag) continue;
        gf = gf + w.dt * contact_force(E, sr.sdf, sr.n, sr.r);
      }
      v3 u = (inv_m * mv + inv_m * gf) + v3{E.dt_g[0], E.dt_g[1], E.dt_g[2]};
      // boundary-condition masks (mpm_elastic.py:227-238)
      const int bd = E.bound;
      bool mx = (i < bd && u.x < 0.f) || (i > E.n[0] - bd && u.x > 0.f);
      bool my = (j < bd && u.y < 0.f) || (j > E.n[1] - bd && u.y > 0.f);
      bool mz = (k < bd && u.z < 0.f) || (k > E.n[2] - bd && u.z > 0.f);
      if (E.bc == DT_BC_STICKY_FLOOR && j < bd) mx = my = mz = true;
      const v3 ub = v3{mx ? 0.f : vb.x, my ? 0.f : vb.y, mz ? 0.f : vb.z};
      v3 mvb = inv_m * ub;
      const v3 gfb = inv_m * ub;
      const float invb = dot(ub, mv + gf);
      float mb = clampg(-inv_m * inv_m * invb, w.grad_clip);  // clamp_grid on grid_m.grad
      // contact adjoint
      v3 curvb = v3{0.f, 0.f, 0.f};
#pragma unroll
      for (int q = 0; q < DT_MAX_SENSORS_PER_ENV; ++q) {
        const int si = E.s_begin + q;
        if (si >= E.s_end) break;
        if (cid[q] < 0) continue;
        const dt_sensor& S = w.sensors[si];
        const int4 tr = __ldg(tris + S.f_off + cid[q]);
        const v3 p1 = f4to3(P[tr.x]), p2 = f4to3(P[tr.y]), p3 = f4to3(P[tr.z]);
        const v3 od = v3{S.out_dir[0], S.out_dir[1], S.out_dir[2]};
        SdfRes sr = find_sdf(p1, p2, p3, f4to3(VM[tr.x]), f4to3(VM[tr.y]), f4to3(VM[tr.z]), od, p, cur_v);
        if (!sr.flag) continue;
        // ext enters grid_f (x dt) and the three sensor vertices (x -1/3)
        const v3 exs = (f4to3(aExt[tr.x]) + f4to3(aExt[tr.y])) + f4to3(aExt[tr.z]);
        const v3 eb = w.dt * gfb - third * exs;
        v3 nb = v3{0.f, 0.f, 0.f}, rb = v3{0.f, 0.f, 0.f};
        const float sdfb = contact_force_bwd(contact_k(E), sr.sdf, sr.n, sr.r, eb, nb, rb);
        // r = mean tri velocity - cur_v
        const v3 tvb = third * rb;
        red_add_v4(aVm + tr.x, v3to4(tvb));
        red_add_v4(aVm + tr.y, v3to4(tvb));
        red_add_v4(aVm + tr.z, v3to4(tvb));
        curvb = curvb - rb;
        v3 b1, b2, b3;
        tri_geom_bwd(p1, p2, p3, od, p, sr.n, sdfb, nb, b1, b2, b3);
        red_add_v4(aPos + tr.x, v3to4(b1));
        red_add_v4(aPos + tr.y, v3to4(b2));
        red_add_v4(aPos + tr.z, v3to4(b3));
      }
      // cur_v = mv / (m + eps)
      mvb = mvb + inv_m * curvb;
      mb += -dot(curvb, mv) * inv_m * inv_m;
      res = make_float4(mvb.x, mvb.y, mvb.z, mb);
    }
    aacc[g] = res;
  }
}

// ---------------------------------------------------------------------------------------------
// B3: P2G + constitutive + SVD adjoint; FEM force adjoint
// ---------------------------------------------------------------------------------------------
__device__ void p2g_bwd(const dt_world& w, int f, int p, float& mub, float& lamb, int& mat) {
  const int nb = (f + 1) & 1, cb = f & 1;
  float4 q[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) q[k] = ldg4(pplane(w, f, k) + p);
  PRec r;
  unpack_rec(q, r);
  // adjoint of F[f+1]
  const float4 n3 = ld4(padj(w, nb, 3) + p), n4 = ld4(padj(w, nb, 4) + p), n5 = ld4(padj(w, nb, 5) + p);
  m3 Fpb;
  Fpb.a[0][0] = n3.w;
  Fpb.a[0][1] = n4.x;
  Fpb.a[0][2] = n4.y;
  Fpb.a[1][0] = n4.z;
  Fpb.a[1][1] = n4.w;
  Fpb.a[1][2] = n5.x;
  Fpb.a[2][0] = n5.y;
  Fpb.a[2][1] = n5.z;
  Fpb.a[2][2] = n5.w;
  const float4 xpart = ld4(padj(w, cb, 0) + p);  // x adjoint from the G2P adjoint
  const dt_env& E = w.envs[__ldg(w.p_env + p)];
  int base[3];
  float fx[3];
  PRec out;
  mat = __ldg(w.p_mat + p);
  mub = lamb = 0.f;
  if (!particle_base(E, r.x, base, fx)) {
    // carried unchanged in the forward pass: adjoint passes straight through
    const float4 a0 = ld4(padj(w, nb, 0) + p), a1 = ld4(padj(w, nb, 1) + p), a2 = ld4(padj(w, nb, 2) + p),
                 a3 = ld4(padj(w, nb, 3) + p);
    float4 o[6] = {make_float4(xpart.x, xpart.y, xpart.z, a0.w), a1, a2, a3, n4, n5};
#pragma unroll
    for (int k = 0; k < 6; ++k) padj(w, cb, k)[p] = o[k];
    return;
  }
  const dt_material M = w.materials[mat];
  Stress s;
  constitutive(r.C, r.F, w.dt, M, w.svd_sweeps, s, &w, w.p_svd ? f : -1, p);  // the forward's SVD if taped
  const float pm = E.p_mass, dx = E.dx;
  m3 A;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) A.a[i][j] = E.stress_k * s.cauchy.a[i][j] + pm * r.C.a[i][j];
  // gather the grid adjoint.  With m_o the momentum adjoint of node o, W_o its weight and
  // dp_o = (o - fx) dx:  v_bar = p_mass S0,  A_bar = dx (S1 - S0 (fx - 1)^T)  with  S0 = sum W_o m_o and
  // S1 = sum W_o m_o (o - 1)^T (the moment about the stencil's middle node),  and
  // fx_bar_d = sum dW_o/dfx_d Wb_o - dx (A^T S0)_d  with
  // Wb_o = m_o . u_o + p_mass mass_bar_o,  u_o = p_mass v + A dp_o = u_1 + sum_c (o_c - 1) a_c
  // (u_1 = p_mass v + A (1 - fx) dx, the middle node's; a_c = dx A column c): the per-node work is two
  // moments, u_o by one add per axis that moves, and Wb_o
  const float4* aacc = reinterpret_cast<const float4*>(w.g_adj_acc);
  v3 S0 = v3{0.f, 0.f, 0.f};
  m3 S1 = mzero();
  float fxb[3] = {0.f, 0.f, 0.f};
  float wts[3][3], dws[3][3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      wts[i][d] = bsw(i, fx[d]);
      dws[i][d] = bsdw(i, fx[d]);
    }
  const v3 a0 = dx * mcol(A, 0), a1 = dx * mcol(A, 1), a2 = dx * mcol(A, 2);
  const v3 u1 = pm * r.v + mvec(A, v3{(1.f - fx[0]) * dx, (1.f - fx[1]) * dx, (1.f - fx[2]) * dx});
  const StencilNodes sn = stencil_nodes(E, base);
  // fx_bar: per row (oi, oj) of three nodes the sums Z = sum_k wz_k Wb and Zd = sum_k dwz_k Wb, then
  // fx_bar += (dwx wy Z, wx dwy Z, wx wy Zd)
#pragma unroll
  for (int oi = 0; oi < 3; ++oi)
#pragma unroll
    for (int oj = 0; oj < 3; ++oj) {
      float Z = 0.f, Zd = 0.f;
#pragma unroll
      for (int ok = 0; ok < 3; ++ok) {
        const v3 ui = oi == 0 ? u1 - a0 : (oi == 1 ? u1 : u1 + a0);  // resolved at compile time
        const v3 uij = oj == 0 ? ui - a1 : (oj == 1 ? ui : ui + a1);
        const v3 u = ok == 0 ? uij - a2 : (ok == 1 ? uij : uij + a2);
        const float4 gb = __ldg(aacc + ((sn.x[oi] + sn.y[oj]) + sn.z[ok]));
        const v3 mvb = f4to3(gb);
        const float W = (wts[oi][0] * wts[oj][1]) * wts[ok][2];
        const v3 Wm = W * mvb;
        S0 = S0 + Wm;
        const float o[3] = {(float)(oi - 1), (float)(oj - 1), (float)(ok - 1)};  // about the middle node
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (o[c] == 0.f) continue;  // resolved at compile time
          S1.a[0][c] += o[c] * Wm.x;
          S1.a[1][c] += o[c] * Wm.y;
          S1.a[2][c] += o[c] * Wm.z;
        }
        const float Wb = dot(mvb, u) + pm * gb.w;
        Z += wts[ok][2] * Wb;
        Zd += dws[ok][2] * Wb;
      }
      fxb[0] += (dws[oi][0] * wts[oj][1]) * Z;
      fxb[1] += (wts[oi][0] * dws[oj][1]) * Z;
      fxb[2] += (wts[oi][0] * wts[oj][1]) * Zd;
    }
  const v3 vb = pm * S0;
  m3 Ab;
#pragma unroll
  for (int rr = 0; rr < 3; ++rr) {
    const float s0 = rr == 0 ? S0.x : (rr == 1 ? S0.y : S0.z);
#pragma unroll
    for (int c = 0; c < 3; ++c) Ab.a[rr][c] = dx * (S1.a[rr][c] - s0 * (fx[c] - 1.f));
  }
  fxb[0] -= dot(a0, S0);  // dx (A^T S0)
  fxb[1] -= dot(a1, S0);
  fxb[2] -= dot(a2, S0);
  // affine = stress_k * cauchy + p_mass * C
  m3 Cb = mscale(pm, Ab);
  const m3 G = mscale(E.stress_k, Ab);  // cauchy adjoint
  m3 Ub = mzero(), Vb = mzero(), Rb = mzero();
  m3 Frm = mzero();  // the return map's rotation-part adjoint when formed directly (von Mises), as
                     // U Frm V^T: added inside the SVD adjoint's final product
  bool uv = false;   // Ub or Vb set (the return map's adjoint through U and V)
  v3 sb = v3{0.f, 0.f, 0.f};
  float Jb;
  if (M.model == DT_MODEL_NEOHOOKEAN) {
    // cauchy = mu (Fp Fp^T - I) + lam log(J) I
    Fpb = madd(Fpb, mscale(M.mu, mmul(madd(G, mT(G)), s.Fp)));
    const float trG = mtrace(G);
    Jb = M.lam * trG / s.J;
    mub = mdot(G, msub(mmulT(s.Fp, s.Fp), meye()));
    lamb = logf(s.J) * trG;
  } else {
    // cauchy = 2 mu (Fp - R) Fp^T + lam J (J - 1) I
    const m3 D = msub(s.Fp, s.R);
    Fpb = madd(Fpb, mscale(2.f * M.mu, madd(mmul(G, s.Fp), mTmul(G, D))));
    Rb = mscale(-2.f * M.mu, mmul(G, s.Fp));  // R = U V^T, handled inside svd_grad
    const float trG = mtrace(G);
    Jb = M.lam * (2.f * s.J - 1.f) * trG;
    mub = 2.f * mdot(G, mmulT(D, s.Fp));
    lamb = s.J * (s.J - 1.f) * trG;
  }
  m3 Fnb;
  if (M.model == DT_MODEL_COROTATED) {
    sb = sb + Jb * v3{s.sig.y * s.sig.z, s.sig.x * s.sig.z, s.sig.x * s.sig.y};
    Fnb = Fpb;
  } else {
    Fpb = madd(Fpb, mscale(Jb, mcof(s.Fp)));  // J = det(Fp)
    if (M.model == DT_MODEL_VON_MISES && s.yield) {
      // Fp = U diag(exp(eps')) V^T (mpm_plastic.py:162-165)
      const float sg[3] = {s.sig.x, s.sig.y, s.sig.z};
      float ep[3], eh[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) ep[d] = logf(fmaxf(sg[d], 0.05f));
      const float mean = ((ep[0] + ep[1]) + ep[2]) / 3.f;
#pragma unroll
      for (int d = 0; d < 3; ++d) eh[d] = ep[d] - mean;
      const float nrm = sqrtf(((eh[0] * eh[0] + eh[1] * eh[1]) + eh[2] * eh[2]) + 1e-8f);
      const float dg = nrm - M.yield_stress / (2.f * M.mu);
      const float rr = dg / nrm;
      float ex[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) ex[d] = expf(ep[d] - rr * eh[d]);
      const m3 UtFV = mmul(mTmul(s.U, Fpb), s.V);
      if (w.svd_grad_mode != DT_SVDGRAD_REFERENCE && sg[0] > 0.05f && sg[1] > 0.05f && sg[2] > 0.05f) {
        // e_k = c s_k^a (a = 1 - rr, c = exp(rr mean)): the rotation part of the SVD adjoint of
        // Fp = U diag(e) V^T has, for i != j and M = U^T Fp_bar V, the entries
        //   M_ij (e_j s_j - e_i s_i) / (s_j^2 - s_i^2) + M_ji (s_i e_j - e_i s_j) / (s_j^2 - s_i^2)
        // = M_ij c dd(a+1) / (s_i + s_j) + M_ji c s_i s_j dd(a-1) / (s_i + s_j),  dd(p) the divided
        // difference of x^p at (s_i, s_j): finite where singular values coincide, unlike the generic
        // formula's 1 / (s_j^2 - s_i^2)
        // (the powers come from e itself: c s^(a+1) = e s, c s^(a-1) = e / s, c s^(a-2) = e / s^2;
        // both factors are symmetric in i, j)
        const float a = 1.f - rr;
        m3 inner = mzero();
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = i + 1; j < 3; ++j) {
            const float sum = sg[i] + sg[j];
            const float A = cdd(sg[i], sg[j], ex[i] * sg[i], ex[j] * sg[j], ex[i], a + 1.f) / sum;
            const float B = (sg[i] * sg[j]) *
                            cdd(sg[i], sg[j], ex[i] / sg[i], ex[j] / sg[j], ex[i] / (sg[i] * sg[i]), a - 1.f) / sum;
            inner.a[i][j] = UtFV.a[i][j] * A + UtFV.a[j][i] * B;
            inner.a[j][i] = UtFV.a[j][i] * A + UtFV.a[i][j] * B;
          }
        Frm = inner;
      } else {
        uv = true;
        m3 Ue = s.U, Ve = s.V;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            Ue.a[i][d] *= ex[d];
            Ve.a[i][d] *= ex[d];
          }
        Ub = madd(Ub, mmul(Fpb, Ve));   // Fpb V diag(e)
        Vb = madd(Vb, mTmul(Fpb, Ue));  // Fpb^T U diag(e)
      }
      float epb[3], ehb[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) epb[d] = UtFV.a[d][d] * ex[d];
      // eps' = eps - rr * eh,  rr = 1 - ys / (2 mu nrm)
      float rrb = 0.f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        ehb[d] = -rr * epb[d];
        rrb -= epb[d] * eh[d];
      }
      const float nrmb = rrb * M.yield_stress / (2.f * M.mu * nrm * nrm);
      mub += rrb * M.yield_stress / (2.f * M.mu * M.mu * nrm);
#pragma unroll
      for (int d = 0; d < 3; ++d) ehb[d] += nrmb * eh[d] / nrm;
      const float mb_ = ((ehb[0] + ehb[1]) + ehb[2]) / 3.f;
      float sbv[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float eb_ = epb[d] + ehb[d] - mb_;
        sbv[d] = sg[d] > 0.05f ? eb_ / sg[d] : 0.f;
      }
      sb = sb + v3{sbv[0], sbv[1], sbv[2]};
      Fnb = mzero();
    } else {
      Fnb = Fpb;
    }
  }
  if (M.model != DT_MODEL_NEOHOOKEAN)
    Fnb = madd(Fnb, svd_grad(s.U, s.sig, s.V, Ub, sb, Vb, Rb, w.svd_grad_mode, uv, Frm));
  // F_new = (I + dt C) F
  m3 Ad = meye();
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Ad.a[i][j] += w.dt * r.C.a[i][j];
  out.F = mTmul(Ad, Fnb);
  Cb = madd(Cb, mscale(w.dt, mmulT(Fnb, r.F)));
  out.C = Cb;
  out.v = vb;
  out.x = v3{xpart.x, xpart.y, xpart.z} + E.inv_dx * v3{fxb[0], fxb[1], fxb[2]};
  float4 o[6];
  pack_rec(out, o);
#pragma unroll
  for (int k = 0; k < 6; ++k) padj(w, cb, k)[p] = o[k];
}

__device__ void fem_tet_bwd(const dt_world& w, int f, int t) {
  const int cb = f & 1;
  const size_t V = (size_t)w.n_verts;
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
  const v3 a = f4to3(P[tv.x]), b = f4to3(P[tv.y]), c = f4to3(P[tv.z]), d = f4to3(P[tv.w]);
  m3 D;
  const v3 cols[3] = {a - d, b - d, c - d};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    D.a[0][k] = cols[k].x;
    D.a[1][k] = cols[k].y;
    D.a[2][k] = cols[k].z;
  }
  const float detD = mdet(D);
  const float Vi = fabsf(detD) / 6.f;
  const m3 Fe = mmul(D, B);
  const float4* aVm0 = reinterpret_cast<const float4*>(w.v_adj_velmid);
  float4* aPos0 = reinterpret_cast<float4*>(w.v_adj_pos) + cb * V;
  if (S.model == DT_FEM_LINEAR_COROTATED) {
    // P = 2 mu (F - R) + lam c R, c = sum sigma - 3, H = -V0 P B^T with the rest volume V0
    m3 U, Vm;
    v3 sg;
    if (w.t_svd)
      load_svd_of(w.t_svd, w.n_tets, f, t, U, sg, Vm);  // the forward's decomposition
    else
      svd3(Fe, U, sg, Vm, w.svd_sweeps);
    const m3 R = mmulT(U, Vm);
    const float c = ((sg.x + sg.y) + sg.z) - 3.f;
    const float sc0 = -S.dt_over_m / (6.f * fabsf(mdet(B)));
    const v3 g3 = f4to3(aVm0[tv.w]);
    const v3 hb[3] = {f4to3(aVm0[tv.x]) - g3, f4to3(aVm0[tv.y]) - g3, f4to3(aVm0[tv.z]) - g3};
    m3 Hb;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      Hb.a[0][k] = sc0 * hb[k].x;
      Hb.a[1][k] = sc0 * hb[k].y;
      Hb.a[2][k] = sc0 * hb[k].z;
    }
    const m3 Pb = mmul(Hb, B);  // H = P B^T
    const m3 Rb = mscale(S.lam * c - 2.f * S.mu, Pb);
    const float cb_ = S.lam * mdot(Pb, R);
    const m3 Fb = madd(mscale(2.f * S.mu, Pb),
                       svd_grad(U, sg, Vm, mzero(), v3{cb_, cb_, cb_}, mzero(), Rb, DT_SVDGRAD_STABLE, false));
    const m3 Db = mmulT(Fb, B);  // F = D B
    const v3 ab = mcol(Db, 0), bb = mcol(Db, 1), cbv = mcol(Db, 2);
    red_add_v4(aPos0 + tv.x, v3to4(ab));
    red_add_v4(aPos0 + tv.y, v3to4(bb));
    red_add_v4(aPos0 + tv.z, v3to4(cbv));
    red_add_v4(aPos0 + tv.w, v3to4(-((ab + bb) + cbv)));
    return;
  }
  const float J = mdet(Fe);
  const float IC = mdot(Fe, Fe);
  const m3 cof = mcof(Fe);
  const float k1 = S.mu * (1.f - 1.f / (IC + 1.f));
  const float k2 = S.lam * (J - S.alpha);
  m3 Pk;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Pk.a[i][j] = k1 * Fe.a[i][j] + k2 * cof.a[i][j];
  const m3 H = mmulT(Pk, B);
  const float sc = -Vi * S.dt_over_m;
  // velocity increments h_k = sc H[:,k] to v_k, -sum to v_3
  const float4* aVm = reinterpret_cast<const float4*>(w.v_adj_velmid);
  const v3 g3 = f4to3(aVm[tv.w]);
  const v3 hb[3] = {f4to3(aVm[tv.x]) - g3, f4to3(aVm[tv.y]) - g3, f4to3(aVm[tv.z]) - g3};
  m3 Hb;
  float scb = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    Hb.a[0][k] = sc * hb[k].x;
    Hb.a[1][k] = sc * hb[k].y;
    Hb.a[2][k] = sc * hb[k].z;
    scb += dot(hb[k], mcol(H, k));
  }
  const float Vib = -S.dt_over_m * scb;
  const m3 Pb = mmul(Hb, B);  // H = P B^T
  // P = k1 F + k2 cof(F)
  m3 Fb = mscale(k1, Pb);
  const float k1b = mdot(Pb, Fe), k2b = mdot(Pb, cof);
  {
    const v3 f0 = mcol(Fe, 0), f1 = mcol(Fe, 1), f2 = mcol(Fe, 2);
    const v3 p0 = mcol(Pb, 0), p1 = mcol(Pb, 1), p2 = mcol(Pb, 2);
    const v3 g0 = cross(p1, f2) + cross(f1, p2);
    const v3 g1 = cross(f2, p0) + cross(p2, f0);
    const v3 g2 = cross(p0, f1) + cross(f0, p1);
    const v3 gg[3] = {g0, g1, g2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      Fb.a[0][k] += k2 * gg[k].x;
      Fb.a[1][k] += k2 * gg[k].y;
      Fb.a[2][k] += k2 * gg[k].z;
    }
  }
  const float ICb = k1b * S.mu / ((IC + 1.f) * (IC + 1.f));
  const float Jb = S.lam * k2b;
  Fb = madd(Fb, madd(mscale(2.f * ICb, Fe), mscale(Jb, cof)));
  m3 Db = mmulT(Fb, B);  // F = D B
  const float sgn = detD < 0.f ? -1.f : (detD > 0.f ? 1.f : 0.f);
  Db = madd(Db, mscale(Vib * sgn / 6.f, mcof(D)));
  const v3 ab = mcol(Db, 0), bb = mcol(Db, 1), cbv = mcol(Db, 2);
  float4* aPos = reinterpret_cast<float4*>(w.v_adj_pos) + cb * V;
  red_add_v4(aPos + tv.x, v3to4(ab));
  red_add_v4(aPos + tv.y, v3to4(bb));
  red_add_v4(aPos + tv.z, v3to4(cbv));
  red_add_v4(aPos + tv.w, v3to4(-((ab + bb) + cbv)));
}

// P2G adjoint of particle p (all 32 lanes of the warp call it: the material grads are summed over
// the warp when it shares one material, then added with one atomic per warp)
__device__ void p2g_bwd_particle(const dt_world& w, int f, int p) {
  float mub = 0.f, lamb = 0.f;
  int mat = -1;
  if (p < w.n_particles) p2g_bwd(w, f, p, mub, lamb, mat);
  const int m0 = __shfl_sync(0xffffffffu, mat, 0);
  const bool same = __all_sync(0xffffffffu, mat == m0 || mat < 0);
  if (same) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mub += __shfl_xor_sync(0xffffffffu, mub, o);
      lamb += __shfl_xor_sync(0xffffffffu, lamb, o);
    }
    if ((threadIdx.x & 31) == 0 && m0 >= 0) {
      atomicAdd(w.mat_adj + 4 * m0 + 0, mub);
      atomicAdd(w.mat_adj + 4 * m0 + 1, lamb);
    }
  } else if (mat >= 0) {
    atomicAdd(w.mat_adj + 4 * mat + 0, mub);
    atomicAdd(w.mat_adj + 4 * mat + 1, lamb);
  }
}

// nb_r > 0: the last nb_r CTAs restore frame f - 1's grid velocities for the next backward substep
// (only stage 1 reads g_vout, so this overlaps stage 3 of frame f)
template <int NT, int PPT>  // DT_MINB_BWD_P2G (4) 128-thread CTAs per SM: 128 registers per thread
__global__ void __launch_bounds__(NT, DT_MINB(DT_MINB_BWD_P2G, NT)) k_bwd_p2g_fem(dt_world w, int f, int nb_p, int nb_t, int nb_v,
                                                             int nb_r) {
  pdl_entry();
  int b = blockIdx.x;
  if (b < nb_p) {
    if (PPT == 1) {
      p2g_bwd_particle(w, f, b * NT + threadIdx.x);
    } else {
      int c0, c1;
      cta_chunks(w, NT, PPT, b, c0, c1);
      for (int c = c0; c < c1; ++c) p2g_bwd_particle(w, f, c * NT + threadIdx.x);
    }
    return;
  }
  b -= nb_p;
  if (b < nb_t) {
    const int t = b * NT + threadIdx.x;
    if (t < w.n_tets) fem_tet_bwd(w, f, t);
    return;
  }
  b -= nb_t;
  if (b < nb_v) {
    const int i = b * NT + threadIdx.x;
    if (i < w.n_verts) {
      reinterpret_cast<float4*>(w.v_adj_vel)[(size_t)(f & 1) * w.n_verts + i] =
          reinterpret_cast<const float4*>(w.v_adj_velmid)[i];
      reinterpret_cast<float4*>(w.v_adj_ext)[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // zero between substeps
    }
    return;
  }
  b -= nb_v;
  if (b < nb_r) restore_blocks(w, f - 1, b, nb_r, NT / 64);
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }
inline int launched() { return launch_status(cudaGetLastError()); }

// stage 1: G2P adjoint (particles) + integration adjoint (vertices)
template <int MODE, int NT, int PPT>
cudaError_t b1_ppt(const dt_world* w, int f, cudaStream_t stream) {
  const int nb_p = particle_ctas(w, NT, PPT), nb_v = cdiv(w->n_verts, NT);
  if (nb_p + nb_v == 0) return cudaSuccess;
  const size_t smem = scatter_smem(MODE, NT);
  return launch_k(k_bwd_g2p_fem<MODE, NT, PPT>, nb_p + nb_v, NT, smem, stream, *w, f, nb_p, nb_v);
}
template <int MODE, int NT>
cudaError_t b1(const dt_world* w, int f, cudaStream_t stream) {
  return per_thread(w) == 2 ? b1_ppt<MODE, NT, 2>(w, f, stream) : b1_ppt<MODE, NT, 1>(w, f, stream);
}

template <int MODE>
cudaError_t b1_nt(const dt_world* w, int f, cudaStream_t stream) {
  switch (particle_block(w)) {
    case 64: return b1<MODE, 64>(w, f, stream);
    case 256: return b1<MODE, 256>(w, f, stream);
    default: return b1<MODE, 128>(w, f, stream);
  }
}

// stage 3: P2G / F adjoint (particles), tet adjoint, vertex hand-over; with `restore`, the last
// CTAs also restore frame f - 1's grid velocities
template <int NT, int PPT>
cudaError_t b3_ppt(const dt_world* w, int f, bool restore, cudaStream_t stream) {
  const int nb_p = particle_ctas(w, NT, PPT), nb_v = cdiv(w->n_verts, NT), nb_t = cdiv(w->n_tets, NT);
  const int per = NT / 64;  // 64-node blocks a restoring CTA copies per pass
  const int nb_r = !restore ? 0 : (w->n_blocks < 152 * 4 * per ? cdiv(w->n_blocks, per) : 152 * 4);
  if (nb_p + nb_t + nb_v + nb_r == 0) return cudaSuccess;
  return launch_k(k_bwd_p2g_fem<NT, PPT>, nb_p + nb_t + nb_v + nb_r, NT, 0, stream, *w, f, nb_p, nb_t, nb_v, nb_r);
}
template <int NT>
cudaError_t b3_nt(const dt_world* w, int f, bool restore, cudaStream_t stream) {
  return per_thread(w) == 2 ? b3_ppt<NT, 2>(w, f, restore, stream) : b3_ppt<NT, 1>(w, f, restore, stream);
}
cudaError_t b3(const dt_world* w, int f, bool restore, cudaStream_t stream) {
  switch (particle_block(w)) {
    case 64: return b3_nt<64>(w, f, restore, stream);
    case 256: return b3_nt<256>(w, f, restore, stream);
    default: return b3_nt<128>(w, f, restore, stream);
  }
}

}  // namespace

extern "C" {

int dt_substep_bwd_stage(const dt_world* w, int f, int stage, cudaStream_t stream) {
  if (!w || f < 0 || f + 1 >= w->n_frames || stage < 0 || stage > 3) return DT_ERR_ARG;
  cudaError_t e = cudaSuccess;
  switch (stage) {
    case 0: {
      const int ng = w->n_blocks < 152 * 16 ? w->n_blocks : 152 * 16;
      if (ng > 0) e = launch_k(k_bwd_restore, ng, GRID_NT, 0, stream, *w, f);
      break;
    }
    case 1:
      switch (scatter_kind_adj(w)) {
        case DT_SCATTER_TILE: e = b1<DT_SCATTER_TILE, NT_TILE>(w, f, stream); break;
        case DT_SCATTER_GLOBAL: e = b1_nt<DT_SCATTER_GLOBAL>(w, f, stream); break;
        case DT_SCATTER_WARP + 1: e = b1_nt<DT_SCATTER_WARP + 1>(w, f, stream); break;
        case DT_SCATTER_WARP + 2: e = b1_nt<DT_SCATTER_WARP + 2>(w, f, stream); break;
        case DT_MODE_SMEM: e = b1_nt<DT_MODE_SMEM>(w, f, stream); break;
        default: e = b1_nt<DT_SCATTER_WARP>(w, f, stream);
      }
      break;
    case 2: {
      const int ng = w->n_blocks < 152 * 16 ? w->n_blocks : 152 * 16;
      if (ng > 0) e = launch_k(k_bwd_grid, ng, GRID_NT, 0, stream, *w, f);
      if (e != cudaSuccess) return DT_ERR_LAUNCH;
      return dt_rope_update_bwd(w, f, stream);
    }
    default:
      e = b3(w, f, false, stream);
  }
  return e == cudaSuccess ? DT_OK : DT_ERR_LAUNCH;
}

int dt_substeps_bwd(const dt_world* w, int f_hi, int f_lo, cudaStream_t stream) {
  if (!w || f_lo < 0 || f_hi <= f_lo || f_hi >= w->n_frames) return DT_ERR_ARG;
  int rc = dt_substep_bwd_stage(w, f_hi - 1, 0, stream);
  if (w->n_ropes > 0 && has_aux(w)) {
    // The solver's adjoint of frame f reads only the rope adjoint of frame f + 1, complete once the rope
    // contact adjoint of f + 1 has run: it runs on the aux stream beside stage 3 of f + 1 and stages 1
    // and the grid adjoint of f, and the contact adjoint of f (which reads its output) waits for it.
    // Work forked onto the aux stream is joined back before the call returns, on errors too.
    bool pending = false;
    auto fork_solve = [&](int g) {
      if (aux_fork(w, stream) != cudaSuccess) return DT_ERR_LAUNCH;
      pending = true;
      return rope_part(w, g, ROPE_SOLVE_BWD, w->aux_stream);
    };
    if (!rc) rc = fork_solve(f_hi - 1);
    const int ng = w->n_blocks < 152 * 16 ? w->n_blocks : 152 * 16;
    for (int f = f_hi - 1; f >= f_lo && !rc; --f) {
      if ((rc = dt_substep_bwd_stage(w, f, 1, stream))) break;
      if (ng > 0 && launch_k(k_bwd_grid, ng, GRID_NT, 0, stream, *w, f) != cudaSuccess) {
        rc = DT_ERR_LAUNCH;
        break;
      }
      pending = false;
      if (aux_join(w, stream) != cudaSuccess) {
        rc = DT_ERR_LAUNCH;
        break;
      }
      if ((rc = rope_part(w, f, ROPE_CONTACT_BWD, stream))) break;
      if (f > f_lo && (rc = fork_solve(f - 1))) break;
      if (b3(w, f, f > f_lo, stream) != cudaSuccess) rc = DT_ERR_LAUNCH;
    }
    if (pending && aux_join(w, stream) != cudaSuccess && !rc) rc = DT_ERR_LAUNCH;
    return rc;
  }
  for (int f = f_hi - 1; f >= f_lo && !rc; --f) {
    if ((rc = dt_substep_bwd_stage(w, f, 1, stream)) || (rc = dt_substep_bwd_stage(w, f, 2, stream))) break;
    // the next (lower) frame's restore rides along
    if (b3(w, f, f > f_lo, stream) != cudaSuccess) rc = DT_ERR_LAUNCH;
  }
  return rc;
}

int dt_substep_bwd(const dt_world* w, int f, cudaStream_t stream) {
  if (!w || f < 0 || f + 1 >= w->n_frames) return DT_ERR_ARG;
  for (int s = 0; s < 4; ++s) {
    const int rc = dt_substep_bwd_stage(w, f, s, stream);
    if (rc) return rc;
  }
  return DT_OK;
}

}  // extern "C"
