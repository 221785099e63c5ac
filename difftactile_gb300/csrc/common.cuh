// Device helpers shared by the forward and adjoint substep kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "difftactile_gb300.h"  // include/ is on the compiler include path

#define DT_DEV __device__ __forceinline__

// Minimum resident CTAs per SM of the particle kernels, stated for 128-thread CTAs (the register cap
// follows: 65536 / (128 * n)); 0 leaves the register count to the compiler.  Measured on the
// 64-environment population (one forward + backward substep at mid-rollout): capping the forward P2G
// at 72 registers (from 80; 44-84 B of spills), G2P at 64 (from 72), the G2P adjoint at 80 (from 96)
// and the grid adjoint at 64 (from 96) raises the resident warps enough to take the substep from 3.50
// to 2.97 ms; a 64-register forward P2G times the same as 72 with more spills
#ifndef DT_MINB_FWD_P2G
#define DT_MINB_FWD_P2G 7
#endif
#ifndef DT_MINB_FWD_G2P
#define DT_MINB_FWD_G2P 8
#endif
#ifndef DT_MINB_BWD_G2P
#define DT_MINB_BWD_G2P 6
#endif
#ifndef DT_MINB_BWD_GRID
#define DT_MINB_BWD_GRID 8
#endif
// the P2G adjoint: 4 CTAs of 128 threads (128 registers; 86 B of spill stores with one particle per
// thread, 178 B with two; 168 registers would hold it without spills).  Measured on the
// re-binned population at mid-rollout: 5 CTAs (96 registers, ~1 KB of spills) 616 -> 772 us; keeping
// the constitutive state out of registers across the 27-node gather (recomputed from the SVD tape
// after it: 48 B of spills) 627 -> 657 us at 4 CTAs, 631 us at 5
// the grid kernel: minimum resident CTAs per SM stated for its 256-thread (4-lane) form, halved for
// the 512-thread (8-lane) form; 4: 64 registers.  Measured on the population substep: 5 (48 registers,
// 260 B of spills) 217 -> 222 us, 6 (40 registers) 238 us
#ifndef DT_MINB_FWD_GRID
#define DT_MINB_FWD_GRID 4
#endif
#ifndef DT_MINB_BWD_P2G
#define DT_MINB_BWD_P2G 4
#endif
// Contact searches over sensors of more than this many groups of 32 centroids first reduce the groups to
// the candidates of the query block (contact.cuh: block_candidates); smaller sensors keep every group's
// box distance in registers.  At most 32 (the register cache's size).
#ifndef DT_CAND_MIN_GROUPS
#define DT_CAND_MIN_GROUPS 32
#endif
// the launch-bounds minimum of a CTA of NT threads for a per-128-thread minimum n
#define DT_MINB(n, NT) ((n) > 0 ? ((n) * 128 + (NT) - 1) / (NT) : 1)

// ------------------------------------------------------------------------------------------
// small fixed-size linear algebra, row-major, fully unrolled into registers
// ------------------------------------------------------------------------------------------
struct m3 {
  float a[3][3];
};
struct v3 {
  float x, y, z;
};

DT_DEV v3 mk3(float x, float y, float z) { return v3{x, y, z}; }
DT_DEV v3 operator+(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
DT_DEV v3 operator-(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
DT_DEV v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
DT_DEV v3 operator*(float s, v3 a) { return v3{s * a.x, s * a.y, s * a.z}; }
DT_DEV v3 operator*(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
DT_DEV v3 operator/(v3 a, float s) { return v3{a.x / s, a.y / s, a.z / s}; }
DT_DEV float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
DT_DEV v3 cross(v3 a, v3 b) { return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
DT_DEV v3 f4to3(float4 a) { return v3{a.x, a.y, a.z}; }
DT_DEV float4 v3to4(v3 a, float w = 0.f) { return make_float4(a.x, a.y, a.z, w); }
DT_DEV float get(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

DT_DEV m3 meye() {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = (i == j) ? 1.f : 0.f;
  return r;
}
DT_DEV m3 mzero() {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = 0.f;
  return r;
}
DT_DEV m3 mmul(const m3& x, const m3& y) {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j] + x.a[i][2] * y.a[2][j];
  return r;
}
// x * y^T
DT_DEV m3 mmulT(const m3& x, const m3& y) {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][0] * y.a[j][0] + x.a[i][1] * y.a[j][1] + x.a[i][2] * y.a[j][2];
  return r;
}
// x^T * y
DT_DEV m3 mTmul(const m3& x, const m3& y) {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[0][i] * y.a[0][j] + x.a[1][i] * y.a[1][j] + x.a[2][i] * y.a[2][j];
  return r;
}
DT_DEV m3 mT(const m3& x) {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[j][i];
  return r;
}
DT_DEV m3 madd(const m3& x, const m3& y) {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] + y.a[i][j];
  return r;
}
DT_DEV m3 msub(const m3& x, const m3& y) {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] - y.a[i][j];
  return r;
}
DT_DEV m3 mscale(float s, const m3& x) {
  m3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[i][j] = s * x.a[i][j];
  return r;
}
DT_DEV float mdot(const m3& x, const m3& y) {
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s += x.a[i][j] * y.a[i][j];
  return s;
}
DT_DEV float mtrace(const m3& x) { return x.a[0][0] + x.a[1][1] + x.a[2][2]; }
DT_DEV float mdet(const m3& m) {
  const float(*a)[3] = m.a;
  return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}
// cofactor matrix: d det(m) / d m
DT_DEV m3 mcof(const m3& m) {
  const float(*a)[3] = m.a;
  m3 c;
  c.a[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  c.a[0][1] = a[1][2] * a[2][0] - a[1][0] * a[2][2];
  c.a[0][2] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  c.a[1][0] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
  c.a[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
  c.a[1][2] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
  c.a[2][0] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
  c.a[2][1] = a[0][2] * a[1][0] - a[0][0] * a[1][2];
  c.a[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
  return c;
}
DT_DEV v3 mcol(const m3& m, int j) { return v3{m.a[0][j], m.a[1][j], m.a[2][j]}; }
DT_DEV v3 mvec(const m3& m, v3 v) {
  return v3{m.a[0][0] * v.x + m.a[0][1] * v.y + m.a[0][2] * v.z, m.a[1][0] * v.x + m.a[1][1] * v.y + m.a[1][2] * v.z,
            m.a[2][0] * v.x + m.a[2][1] * v.y + m.a[2][2] * v.z};
}
DT_DEV v3 mTvec(const m3& m, v3 v) {
  return v3{m.a[0][0] * v.x + m.a[1][0] * v.y + m.a[2][0] * v.z, m.a[0][1] * v.x + m.a[1][1] * v.y + m.a[2][1] * v.z,
            m.a[0][2] * v.x + m.a[1][2] * v.y + m.a[2][2] * v.z};
}

// ------------------------------------------------------------------------------------------
// 3x3 SVD, convention of ti.svd: A = U diag(s) V^T with det U = det V = +1, |s0| >= |s1| >= |s2|,
// s0, s1 >= 0, s2 signed.  Published method: cyclic Jacobi on A^T A with the classical rotation
// (Golub & Van Loan, Matrix Computations, Alg. 8.4.1), columns of A V sorted by norm with a
// sign flip per swap, then Givens QR — the outline of McAdams et al. 2011 ("Computing the SVD
// of 3x3 matrices with minimal branching and elementary floating point operations") with exact
// rotation angles.
// ------------------------------------------------------------------------------------------
// Correctly rounded divisions and square roots in the rotations: with approximate reciprocals the
// factors reconstruct F only to ~2e-7, which the corotated stress 2 mu (F - R) F^T of a stiff material
// near F = I amplifies (E = 4e5, F - R ~ 0.05: 1e-5 relative in the grid momentum; 6e-6 with these)
// One Jacobi rotation of the symmetric S = A^T A in the (p, q) plane, on its six distinct entries:
// app, aqq, apq and the third row's arp, arq (r the index other than p, q).  The rotation angle is the
// classical one, cot 2theta = (aqq - app) / (2 apq) with the smaller tangent; the update is the
// symmetric form of J^T S J (Golub & Van Loan, "Matrix Computations", 4th ed., sec. 8.5.2; Rutishauser
// 1966): app - t apq, aqq + t apq, apq = 0 exactly, and the third row rotated — 6 products instead of
// the 24 of the two-sided update; V accumulates the rotations.
DT_DEV void jacobi_rot(float& app, float& aqq, float& apq, float& arp, float& arq, float V[3][3], int p, int q) {
  if (apq == 0.f) return;
  const float tau = (aqq - app) / (2.f * apq);
  const float t = (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.f)));
  const float c = 1.f / sqrtf(fmaf(t, t, 1.f));
  const float s = t * c;
  app = fmaf(-t, apq, app);
  aqq = fmaf(t, apq, aqq);
  apq = 0.f;
  const float rp = arp, rq = arq;
  arp = c * rp - s * rq;
  arq = s * rp + c * rq;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float vp = V[k][p], vq = V[k][q];
    V[k][p] = c * vp - s * vq;
    V[k][q] = s * vp + c * vq;
  }
}

DT_DEV void swap_cols_neg(float B[3][3], float V[3][3], int i, int j) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float b = B[k][i];
    B[k][i] = B[k][j];
    B[k][j] = -b;
    float v = V[k][i];
    V[k][i] = V[k][j];
    V[k][j] = -v;
  }
}

DT_DEV void qr_givens(float B[3][3], float U[3][3], int i, int j, int col) {
  float a = B[i][col], b = B[j][col];
  float r2 = a * a + b * b;
  float c = 1.f, s = 0.f;
  if (r2 > 1e-30f) {
    const float ir = 1.f / sqrtf(r2);
    c = a * ir;
    s = b * ir;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float bi = B[i][k], bj = B[j][k];
    B[i][k] = c * bi + s * bj;
    B[j][k] = -s * bi + c * bj;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float ui = U[k][i], uj = U[k][j];
    U[k][i] = c * ui + s * uj;
    U[k][j] = -s * ui + c * uj;
  }
}

// columns of M made orthonormal in order (modified Gram-Schmidt); a rotation stays a rotation
DT_DEV void orthonormalize(float M[3][3]) {
  float n0 = rsqrtf(M[0][0] * M[0][0] + M[1][0] * M[1][0] + M[2][0] * M[2][0]);
#pragma unroll
  for (int i = 0; i < 3; ++i) M[i][0] *= n0;
  float d01 = M[0][0] * M[0][1] + M[1][0] * M[1][1] + M[2][0] * M[2][1];
#pragma unroll
  for (int i = 0; i < 3; ++i) M[i][1] -= d01 * M[i][0];
  float n1 = rsqrtf(M[0][1] * M[0][1] + M[1][1] * M[1][1] + M[2][1] * M[2][1]);
#pragma unroll
  for (int i = 0; i < 3; ++i) M[i][1] *= n1;
  float d02 = M[0][0] * M[0][2] + M[1][0] * M[1][2] + M[2][0] * M[2][2];
  float d12 = M[0][1] * M[0][2] + M[1][1] * M[1][2] + M[2][1] * M[2][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) M[i][2] -= d02 * M[i][0] + d12 * M[i][1];
  float n2 = rsqrtf(M[0][2] * M[0][2] + M[1][2] * M[1][2] + M[2][2] * M[2][2]);
#pragma unroll
  for (int i = 0; i < 3; ++i) M[i][2] *= n2;
}

DT_DEV void svd3(const m3& A, m3& U, v3& sv, m3& V, int sweeps) {
  // the six distinct entries of S = A^T A
#define DT_ATA(i, j) (A.a[0][i] * A.a[0][j] + A.a[1][i] * A.a[1][j] + A.a[2][i] * A.a[2][j])
  float s00 = DT_ATA(0, 0), s11 = DT_ATA(1, 1), s22 = DT_ATA(2, 2);
  float s01 = DT_ATA(0, 1), s02 = DT_ATA(0, 2), s12 = DT_ATA(1, 2);
#undef DT_ATA
  float Vm[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
  for (int it = 0; it < sweeps; ++it) {
    // converged once the off-diagonal is below fp32 resolution of the diagonal
    const float off = s01 * s01 + s02 * s02 + s12 * s12;
    const float dia = s00 * s00 + s11 * s11 + s22 * s22;
    if (off <= 1e-15f * dia) break;
    jacobi_rot(s00, s11, s01, s02, s12, Vm, 0, 1);  // third row r = 2: (S20, S21) = (s02, s12)
    jacobi_rot(s00, s22, s02, s01, s12, Vm, 0, 2);  // r = 1: (S10, S12) = (s01, s12)
    jacobi_rot(s11, s22, s12, s01, s02, Vm, 1, 2);  // r = 0: (S01, S02) = (s01, s02)
  }
  float B[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B[i][j] = A.a[i][0] * Vm[0][j] + A.a[i][1] * Vm[1][j] + A.a[i][2] * Vm[2][j];
#define DT_CN(j) (B[0][j] * B[0][j] + B[1][j] * B[1][j] + B[2][j] * B[2][j])
  if (DT_CN(0) < DT_CN(1)) swap_cols_neg(B, Vm, 0, 1);
  if (DT_CN(0) < DT_CN(2)) swap_cols_neg(B, Vm, 0, 2);
  if (DT_CN(1) < DT_CN(2)) swap_cols_neg(B, Vm, 1, 2);
#undef DT_CN
  float Um[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
  qr_givens(B, Um, 0, 1, 0);
  qr_givens(B, Um, 0, 2, 0);
  qr_givens(B, Um, 1, 2, 1);
  sv = v3{B[0][0], B[1][1], B[2][2]};
  // one Gram-Schmidt pass on both factors: the rotations' approximate reciprocals leave columns
  // ~1e-6 off orthonormal, which the SVD adjoint's 1 / (s_j^2 - s_i^2) factors amplify wherever two
  // singular values nearly coincide; the pass brings them to rounding (~1e-7)
  orthonormalize(Um);
  orthonormalize(Vm);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      U.a[i][j] = Um[i][j];
      V.a[i][j] = Vm[i][j];
    }
}

// ------------------------------------------------------------------------------------------
// quadratic B-spline (mpm_elastic.py:178-181); weight index i in {0,1,2} selected without
// dynamic register indexing
// ------------------------------------------------------------------------------------------
DT_DEV float bsw(int i, float fx) {
  float a = 1.5f - fx, b = fx - 1.f, c = fx - 0.5f;
  return i == 0 ? 0.5f * (a * a) : (i == 1 ? 0.75f - b * b : 0.5f * (c * c));
}
DT_DEV float bsdw(int i, float fx) { return i == 0 ? fx - 1.5f : (i == 1 ? -2.f * (fx - 1.f) : fx - 0.5f); }

// ------------------------------------------------------------------------------------------
// grid addressing: 4x4x4-node blocks, env-major
// ------------------------------------------------------------------------------------------
DT_DEV int node_index(const dt_env& E, int i, int j, int k) {
  int b = ((i >> 2) * E.nb[1] + (j >> 2)) * E.nb[2] + (k >> 2);
  return E.node_off + (b << 6) + ((i & 3) << 4) + ((j & 3) << 2) + (k & 3);
}
// The 27 node indices of the stencil at `base`, per axis: node_index(E, base + o) = x[o_x] + y[o_y] + z[o_z]
// (the block term ((bi nb1 + bj) nb2 + bk) 64 distributed over the axes), so that a node costs one add
// on the row's x + y instead of the block product
struct StencilNodes {
  int x[3], y[3], z[3];
};
DT_DEV StencilNodes stencil_nodes(int node_off, int nb1, int nb2, const int base[3]) {
  StencilNodes s;
  const int ry = nb2 << 6, rx = nb1 * ry;
#pragma unroll
  for (int o = 0; o < 3; ++o) {
    const int i = base[0] + o, j = base[1] + o, k = base[2] + o;
    s.x[o] = node_off + (i >> 2) * rx + ((i & 3) << 4);
    s.y[o] = (j >> 2) * ry + ((j & 3) << 2);
    s.z[o] = ((k >> 2) << 6) + (k & 3);
  }
  return s;
}
DT_DEV StencilNodes stencil_nodes(const dt_env& E, const int base[3]) {
  return stencil_nodes(E.node_off, E.nb[1], E.nb[2], base);
}
DT_DEV int block_index(const dt_env& E, int bi, int bj, int bk) {
  return E.blk_off + (bi * E.nb[1] + bj) * E.nb[2] + bk;
}

// ------------------------------------------------------------------------------------------
// memory helpers
// ------------------------------------------------------------------------------------------
// Fire-and-forget vector reduction into a global accumulator.  No kernel reads back, in the same
// launch, what its REDs accumulate, so no memory clobber: the compiler may keep loaded values
// (table fields, particle data) in registers across the 27 REDs of a stencil.
DT_DEV void red_add_v4(float4* addr, float4 v) {
  asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z),
               "f"(v.w));
}
DT_DEV float4 ldg4(const float4* p) { return __ldg(p); }
DT_DEV void set_err(const dt_world& w, int bits) { atomicOr(w.err, bits); }

// Programmatic dependent launch.  Kernels of the substep pipeline begin with pdl_entry(): wait
// until the preceding kernel of the stream has completed and its writes are visible, then let the
// next kernel be launched (its CTAs become resident and wait in their own pdl_entry), which hides
// the launch latency between the short dependent kernels of a substep.  Launched without the
// attribute (pdl_flag() == 0) the wait returns at once.
DT_DEV void pdl_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
// The last CUDA error an entry point of the library met on this host thread (dt_last_error).
inline cudaError_t& last_cuda_error() {
  thread_local cudaError_t e = cudaSuccess;
  return e;
}
inline cudaError_t note_error(cudaError_t e) {
  if (e != cudaSuccess) last_cuda_error() = e;
  return e;
}
// DT_OK, or DT_ERR_LAUNCH with the CUDA error kept for dt_last_error
inline int launch_status(cudaError_t e) { return note_error(e) == cudaSuccess ? DT_OK : DT_ERR_LAUNCH; }

// template scatter mode of the particle launches: DT_SCATTER_WARP + scatter_depth (depth 1 or 2)
// (template MODE: DT_SCATTER_TILE, DT_SCATTER_GLOBAL, DT_SCATTER_WARP + depth, DT_MODE_SMEM + depth)
constexpr int DT_MODE_SMEM = 8;
constexpr int DT_SMEM_TILE = 512;  // nodes of the shared-memory tile of the SMEM scatter (8 KB)
inline int scatter_kind(const dt_world* w) {
  const int d = (w->scatter_depth == 1 || w->scatter_depth == 2) ? w->scatter_depth : 0;
  if (w->scatter_mode == DT_SCATTER_SMEM) return DT_MODE_SMEM;  // whole runs only (the fastest SMEM variant)
  if (w->scatter_mode != DT_SCATTER_WARP) return w->scatter_mode == DT_SCATTER_TILE ? DT_SCATTER_TILE : DT_SCATTER_GLOBAL;
  return DT_SCATTER_WARP + d;
}
// template scatter mode of the G2P adjoint's launch: scatter_kind, with the WARP reduction's depth
// taken from scatter_depth_adj when that is 1, 2 or 3 (3: whole runs)
inline int scatter_kind_adj(const dt_world* w) {
  const int k = scatter_kind(w), a = w->scatter_depth_adj;
  if (k < DT_SCATTER_WARP || k > DT_SCATTER_WARP + 2 || a < 1 || a > 3) return k;
  return DT_SCATTER_WARP + (a == 3 ? 0 : a);
}
// dynamic shared memory of a particle-role launch with scatter MODE and NT threads
constexpr size_t scatter_smem(int MODE, int NT) {
  return MODE == DT_SCATTER_TILE ? 25 * NT * sizeof(float) : (MODE >= DT_MODE_SMEM ? DT_SMEM_TILE * 16 : 0);
}
// threads per CTA of the particle / tet / vertex launches (dt_world.p_block)
inline int particle_block(const dt_world* w) { return (w->p_block == 64 || w->p_block == 256) ? w->p_block : 128; }
// The rope stages one at a time (rope.cu): the contact and the solver of dt_rope_update, the solver's
// adjoint and the contact's adjoint of dt_rope_update_bwd.
enum { ROPE_CONTACT = 0, ROPE_SOLVE = 1, ROPE_SOLVE_BWD = 2, ROPE_CONTACT_BWD = 3 };
int rope_part(const dt_world* w, int f, int part, cudaStream_t stream);

// Fork / join of work onto dt_world.aux_stream: fork() makes the aux stream wait for what the call's
// stream has queued so far; join() makes the call's stream wait for what was queued on the aux stream.
inline bool has_aux(const dt_world* w) { return w->aux_stream && w->aux_events[0] && w->aux_events[1]; }
inline cudaError_t aux_fork(const dt_world* w, cudaStream_t st) {
  cudaError_t e = note_error(cudaEventRecord(w->aux_events[0], st));
  return e == cudaSuccess ? note_error(cudaStreamWaitEvent(w->aux_stream, w->aux_events[0], 0)) : e;
}
inline cudaError_t aux_join(const dt_world* w, cudaStream_t st) {
  cudaError_t e = note_error(cudaEventRecord(w->aux_events[1], w->aux_stream));
  return e == cudaSuccess ? note_error(cudaStreamWaitEvent(st, w->aux_events[1], 0)) : e;
}

// particles per thread (dt_world.p_per_thread): PPT consecutive chunks of NT particles per CTA, a
// template parameter of the particle-role kernels (1 or 2) so that the one-chunk kernels keep their
// register allocation
inline int per_thread(const dt_world* w) { return w->p_per_thread == 2 ? 2 : 1; }
// CTAs of a particle-role launch of NT-thread CTAs, PPT chunks each
inline int particle_ctas(const dt_world* w, int NT, int PPT) {
  const int chunks = (w->n_particles + NT - 1) / NT;
  return (chunks + PPT - 1) / PPT;
}
// the chunks [c0, c1) of NT particles that CTA b of a particle-role launch of PPT chunks takes
DT_DEV void cta_chunks(const dt_world& w, int NT, int PPT, int b, int& c0, int& c1) {
  const int chunks = (w.n_particles + NT - 1) / NT;
  c0 = b * PPT;
  c1 = min(chunks, c0 + PPT);
}

// Opt a kernel into more than 48 KB of dynamic shared memory on the current device (the attribute
// is per device; `cache` remembers the largest size already set on each of up to 64 devices).
inline cudaError_t ensure_smem(const void* fn, size_t bytes, size_t (&cache)[64]) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (bytes <= cache[dev]) return cudaSuccess;
  const cudaError_t e = note_error(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  if (e == cudaSuccess) cache[dev] = bytes;
  return e;
}
inline int& pdl_flag() {
  static int on = 1;
  return on;
}
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_flag() ? 1 : 0;
  return note_error(cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...));
}

// particle record access: plane k of frame f
DT_DEV float4* pplane(const dt_world& w, int f, int k) {
  return reinterpret_cast<float4*>(w.p_state) + ((size_t)f * 6 + k) * (size_t)w.n_particles;
}
DT_DEV float4* padj(const dt_world& w, int buf, int k) {
  return reinterpret_cast<float4*>(w.p_adj) + ((size_t)buf * 6 + k) * (size_t)w.n_particles;
}
DT_DEV float4* vframe(float* base, const dt_world& w, int f) {
  return reinterpret_cast<float4*>(base) + (size_t)f * (size_t)w.n_verts;
}

struct PRec {
  v3 x, v;
  m3 C, F;
};

DT_DEV void unpack_rec(const float4 q[6], PRec& r) {
  r.x = v3{q[0].x, q[0].y, q[0].z};
  r.v = v3{q[0].w, q[1].x, q[1].y};
  r.C.a[0][0] = q[1].z;
  r.C.a[0][1] = q[1].w;
  r.C.a[0][2] = q[2].x;
  r.C.a[1][0] = q[2].y;
  r.C.a[1][1] = q[2].z;
  r.C.a[1][2] = q[2].w;
  r.C.a[2][0] = q[3].x;
  r.C.a[2][1] = q[3].y;
  r.C.a[2][2] = q[3].z;
  r.F.a[0][0] = q[3].w;
  r.F.a[0][1] = q[4].x;
  r.F.a[0][2] = q[4].y;
  r.F.a[1][0] = q[4].z;
  r.F.a[1][1] = q[4].w;
  r.F.a[1][2] = q[5].x;
  r.F.a[2][0] = q[5].y;
  r.F.a[2][1] = q[5].z;
  r.F.a[2][2] = q[5].w;
}
DT_DEV void pack_rec(const PRec& r, float4 q[6]) {
  q[0] = make_float4(r.x.x, r.x.y, r.x.z, r.v.x);
  q[1] = make_float4(r.v.y, r.v.z, r.C.a[0][0], r.C.a[0][1]);
  q[2] = make_float4(r.C.a[0][2], r.C.a[1][0], r.C.a[1][1], r.C.a[1][2]);
  q[3] = make_float4(r.C.a[2][0], r.C.a[2][1], r.C.a[2][2], r.F.a[0][0]);
  q[4] = make_float4(r.F.a[0][1], r.F.a[0][2], r.F.a[1][0], r.F.a[1][1]);
  q[5] = make_float4(r.F.a[1][2], r.F.a[2][0], r.F.a[2][1], r.F.a[2][2]);
}

DT_DEV bool finite3(v3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

// B-spline base cell: truncation toward zero like Taichi's cast(int) (mpm_elastic.py:178)
DT_DEV bool particle_base(const dt_env& E, v3 x, int base[3], float fx[3]) {
  float g0 = x.x * E.inv_dx - 0.5f, g1 = x.y * E.inv_dx - 0.5f, g2 = x.z * E.inv_dx - 0.5f;
  bool ok = (g0 == g0) && (g1 == g1) && (g2 == g2) && fabsf(g0) < 1e6f && fabsf(g1) < 1e6f && fabsf(g2) < 1e6f;
  base[0] = ok ? (int)g0 : 0;
  base[1] = ok ? (int)g1 : 0;
  base[2] = ok ? (int)g2 : 0;
  fx[0] = x.x * E.inv_dx - (float)base[0];
  fx[1] = x.y * E.inv_dx - (float)base[1];
  fx[2] = x.z * E.inv_dx - (float)base[2];
#pragma unroll
  for (int d = 0; d < 3; ++d) ok = ok && base[d] >= 0 && base[d] + 2 < E.n[d];
  return ok;
}

// ------------------------------------------------------------------------------------------
// constitutive model of one particle (shared by P2G and its adjoint)
// ------------------------------------------------------------------------------------------
struct Stress {
  m3 Fn, U, V, Fp, R, cauchy;
  v3 sig;
  float J;
  bool yield;
};

// von Mises return mapping (mpm_plastic.py:151-166); F unchanged unless yielding
DT_DEV void von_mises(Stress& s, float mu, float ys) {
  float e0 = logf(fmaxf(s.sig.x, 0.05f)), e1 = logf(fmaxf(s.sig.y, 0.05f)), e2 = logf(fmaxf(s.sig.z, 0.05f));
  float mean = ((e0 + e1) + e2) / 3.f;
  float h0 = e0 - mean, h1 = e1 - mean, h2 = e2 - mean;
  float nrm = sqrtf(((h0 * h0 + h1 * h1) + h2 * h2) + 1e-8f);
  float dg = nrm - ys / (2.f * mu);
  s.yield = dg > 0.f;
  if (s.yield) {
    float r = dg / nrm;
    float x0 = expf(e0 - r * h0), x1 = expf(e1 - r * h1), x2 = expf(e2 - r * h2);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        s.Fp.a[i][j] = s.U.a[i][0] * x0 * s.V.a[j][0] + s.U.a[i][1] * x1 * s.V.a[j][1] + s.U.a[i][2] * x2 * s.V.a[j][2];
  } else {
    s.Fp = s.Fn;
  }
}

// the SVD of F_new as stored on the tape: 6 float4 planes per particle and frame,
// (U00 U01 U02 U10) (U11 U12 U20 U21) (U22 V00 V01 V02) (V10 V11 V12 V20) (V21 V22 s0 s1) (s2 y 0 0)
// with y = 1 where the von Mises return map yielded (the branch its adjoint differentiates), else 0
// (the tets' tape t_svd has the same planes over n_tets)
DT_DEV float4* svd_plane_of(float* base, int n, int f, int k) {
  return reinterpret_cast<float4*>(base) + ((size_t)f * 6 + k) * (size_t)n;
}
DT_DEV float4* svd_plane(const dt_world& w, int f, int k) { return svd_plane_of(w.p_svd, w.n_particles, f, k); }
DT_DEV void store_svd_of(float* base, int n, int f, int p, const m3& U, v3 sg, const m3& V, bool yield) {
  svd_plane_of(base, n, f, 0)[p] = make_float4(U.a[0][0], U.a[0][1], U.a[0][2], U.a[1][0]);
  svd_plane_of(base, n, f, 1)[p] = make_float4(U.a[1][1], U.a[1][2], U.a[2][0], U.a[2][1]);
  svd_plane_of(base, n, f, 2)[p] = make_float4(U.a[2][2], V.a[0][0], V.a[0][1], V.a[0][2]);
  svd_plane_of(base, n, f, 3)[p] = make_float4(V.a[1][0], V.a[1][1], V.a[1][2], V.a[2][0]);
  svd_plane_of(base, n, f, 4)[p] = make_float4(V.a[2][1], V.a[2][2], sg.x, sg.y);
  svd_plane_of(base, n, f, 5)[p] = make_float4(sg.z, yield ? 1.f : 0.f, 0.f, 0.f);
}
DT_DEV void store_svd(const dt_world& w, int f, int p, const m3& U, v3 sg, const m3& V, bool yield) {
  store_svd_of(w.p_svd, w.n_particles, f, p, U, sg, V, yield);
}
DT_DEV void load_svd_of(float* base, int n, int f, int p, m3& U, v3& sg, m3& V) {
  const float4 a = svd_plane_of(base, n, f, 0)[p], b = svd_plane_of(base, n, f, 1)[p],
               c = svd_plane_of(base, n, f, 2)[p], d = svd_plane_of(base, n, f, 3)[p],
               e = svd_plane_of(base, n, f, 4)[p], g = svd_plane_of(base, n, f, 5)[p];
  U.a[0][0] = a.x; U.a[0][1] = a.y; U.a[0][2] = a.z; U.a[1][0] = a.w;
  U.a[1][1] = b.x; U.a[1][2] = b.y; U.a[2][0] = b.z; U.a[2][1] = b.w;
  U.a[2][2] = c.x; V.a[0][0] = c.y; V.a[0][1] = c.z; V.a[0][2] = c.w;
  V.a[1][0] = d.x; V.a[1][1] = d.y; V.a[1][2] = d.z; V.a[2][0] = d.w;
  V.a[2][1] = e.x; V.a[2][2] = e.y; sg = v3{e.z, e.w, g.x};
}
DT_DEV void load_svd(const dt_world& w, int f, int p, m3& U, v3& sg, m3& V) {
  load_svd_of(w.p_svd, w.n_particles, f, p, U, sg, V);
}

// constitutive update of one particle (compute_new_F + svd + stress, mpm_elastic.py:135-187,
// mpm_plastic.py:151-166,228-235).  svd_src: frame whose tape holds the SVD of this F_new (the
// backward re-reading the forward's), or -1 to compute it.  Neo-Hookean stress needs no SVD.
DT_DEV void constitutive(const m3& C, const m3& F, float dt, const dt_material& M, int sweeps, Stress& s,
                         const dt_world* w = nullptr, int svd_src = -1, int p = 0) {
  m3 A = meye();
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) A.a[i][j] += dt * C.a[i][j];
  s.Fn = mmul(A, F);  // compute_new_F, mpm_elastic.py:137
  if (M.model == DT_MODEL_NEOHOOKEAN) {
    s.U = meye();
    s.V = meye();
    s.sig = v3{1.f, 1.f, 1.f};
  } else if (w != nullptr && svd_src >= 0) {
    load_svd(*w, svd_src, p, s.U, s.sig, s.V);
  } else {
    svd3(s.Fn, s.U, s.sig, s.V, sweeps);
  }
  s.R = mmulT(s.U, s.V);
  s.yield = false;
  if (M.model == DT_MODEL_VON_MISES) {
    von_mises(s, M.mu, M.yield_stress);
    s.J = mdet(s.Fp);
  } else if (M.model == DT_MODEL_NEOHOOKEAN) {
    s.Fp = s.Fn;
    s.J = mdet(s.Fp);
  } else {
    s.Fp = s.Fn;
    s.J = s.sig.x * (s.sig.y * s.sig.z);
  }
  if (M.model == DT_MODEL_NEOHOOKEAN) {
    m3 FFt = mmulT(s.Fp, s.Fp);
    float lj = M.lam * logf(s.J);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) s.cauchy.a[i][j] = M.mu * (FFt.a[i][j] - (i == j ? 1.f : 0.f)) + (i == j ? lj : 0.f);
  } else {
    m3 DFt = mmulT(msub(s.Fp, s.R), s.Fp);
    float lj = M.lam * s.J * (s.J - 1.f);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) s.cauchy.a[i][j] = 2.f * M.mu * DFt.a[i][j] + (i == j ? lj : 0.f);
  }
}

// ------------------------------------------------------------------------------------------
// contact geometry (find_sdf, fem_sensor.py:362-394) and force (grasp_plastic.py:205-216)
// ------------------------------------------------------------------------------------------
struct SdfRes {
  float sdf;
  v3 n;    // plane normal oriented by out_dir (= -norm_v)
  v3 r;    // triangle mean velocity - node velocity (= -relative_v)
  bool flag;
};

// find_sdf, fem_sensor.py:362-394; `offset` is the PBD collision offset (:387-388), subtracted after
// the projection
DT_DEV SdfRes find_sdf(v3 p1, v3 p2, v3 p3, v3 va, v3 vb, v3 vc, v3 od, v3 p, v3 gv, float offset = 0.f) {
  v3 e1 = p2 - p1, e2 = p3 - p1;
  v3 n = cross(e1, e2);
  float len = sqrtf(dot(n, n));
  n = (1.f / (len + 1e-10f)) * n;
  float sg = dot(n, od) < 0.f ? -1.f : 1.f;
  n = sg * n;
  float sdf = dot(p - p1, n);
  v3 proj = p - sdf * n;
  v3 v0 = p3 - p1, v1 = p2 - p1, v2 = proj - p1;
  float d00 = dot(v0, v0), d01 = dot(v0, v1), d02 = dot(v0, v2), d11 = dot(v1, v1), d12 = dot(v1, v2);
  float invd = 1.f / (d00 * d11 - d01 * d01);
  float u = (d11 * d02 - d01 * d12) * invd;
  float v = (d00 * d12 - d01 * d02) * invd;
  const float third = 1.f / 3.f;
  v3 tv = third * ((va + vb) + vc);
  SdfRes o;
  sdf -= offset;
  o.sdf = sdf;
  o.n = n;
  o.r = tv - gv;
  o.flag = sdf < 0.f && u >= 0.f && v >= 0.f && (u + v <= 1.f);
  return o;
}

// penalty + Coulomb-capped friction contact (calculate_contact_force): grasp_plastic.py:205-216
// clamps the normal approach speed at 0 (clamp_vn), cable_straightening.py:212-224 does not
struct ContactK {
  float kn, kd, kt, mu_t;
  bool clamp_vn;
};
DT_DEV ContactK contact_k(const dt_env& E) { return ContactK{E.kn, E.kd, E.kt, E.mu_t, true}; }

DT_DEV v3 contact_force(const ContactK& K, float sdf, v3 n, v3 r) {
  float nr = dot(n, r);
  float vn = K.clamp_vn ? fmaxf(nr, 0.f) : nr;
  float kk = K.kn + K.kd * vn;
  v3 fn = (-kk * sdf) * n;
  v3 vt = r - nr * n;
  float vtn = sqrtf(dot(vt, vt) + 1e-11f);
  v3 ft = v3{0.f, 0.f, 0.f};
  if (vtn > 1e-4f) {
    float g = fminf(K.kt * vtn, K.mu_t * sqrtf(dot(fn, fn)));
    ft = v3{(vt.x / vtn) * g, (vt.y / vtn) * g, (vt.z / vtn) * g};
  }
  return fn + ft;
}
DT_DEV v3 contact_force(const dt_env& E, float sdf, v3 n, v3 r) { return contact_force(contact_k(E), sdf, n, r); }

// adjoint of contact_force: returns sdf_b, accumulates n_b and r_b
DT_DEV float contact_force_bwd(const ContactK& K, float sdf, v3 n, v3 r, v3 eb, v3& nb, v3& rb) {
  const float nr = dot(n, r);
  const float vn = K.clamp_vn ? fmaxf(nr, 0.f) : nr;
  const float kk = K.kn + K.kd * vn;
  const v3 fn = (-kk * sdf) * n;
  const v3 vt = r - nr * n;
  const float vtn = sqrtf(dot(vt, vt) + 1e-11f);
  v3 fnb = eb;
  v3 vtb = v3{0.f, 0.f, 0.f};
  if (vtn > 1e-4f) {
    const float fnn = sqrtf(dot(fn, fn));
    const float kv = K.kt * vtn, cap = K.mu_t * fnn;
    const float g = fminf(kv, cap);
    const v3 th = (1.f / vtn) * vt;
    const float gb = dot(th, eb);
    const v3 thb = g * eb;
    float vtnb = 0.f;
    if (kv <= cap) {
      vtnb += K.kt * gb;
    } else if (fnn > 0.f) {
      fnb = fnb + (K.mu_t * gb / fnn) * fn;
    }
    vtb = (1.f / vtn) * thb;
    vtnb += -dot(thb, vt) / (vtn * vtn);
    vtb = vtb + (vtnb / vtn) * vt;
  }
  // vt = r - nr n
  rb = rb + vtb;
  float nrb = -dot(n, vtb);
  nb = nb - nr * vtb;
  // fn = -kk sdf n
  const float nfb = dot(n, fnb);
  const float kkb = -sdf * nfb;
  const float sdfb = -kk * nfb;
  nb = nb - (kk * sdf) * fnb;
  const float vnb = K.kd * kkb;
  if (!K.clamp_vn || nr > 0.f) nrb += vnb;
  nb = nb + nrb * r;
  rb = rb + nrb * n;
  return sdfb;
}

// adjoint of the triangle geometry in find_sdf for a contact at p (sdf = (p - p1) . n,
// n = sg cross(p2 - p1, p3 - p1) / (|.| + 1e-10)): vertex position adjoints b1, b2, b3
DT_DEV void tri_geom_bwd(v3 p1, v3 p2, v3 p3, v3 od, v3 p, v3 n, float sdfb, v3 nb, v3& b1, v3& b2, v3& b3) {
  v3 p1b = -sdfb * n;
  nb = nb + sdfb * (p - p1);
  const v3 e1 = p2 - p1, e2 = p3 - p1;
  const v3 nrm = cross(e1, e2);
  const float L = sqrtf(dot(nrm, nrm));
  const float sg = dot((1.f / (L + 1e-10f)) * nrm, od) < 0.f ? -1.f : 1.f;
  v3 nrmb = v3{0.f, 0.f, 0.f};
  if (L > 0.f) {
    const float D = L + 1e-10f;
    nrmb = sg * ((1.f / D) * nb - (dot(nb, nrm) / (D * D * L)) * nrm);
  }
  b2 = cross(e2, nrmb);
  b3 = cross(nrmb, e1);
  b1 = p1b - (b2 + b3);
}

// ------------------------------------------------------------------------------------------
// Privatised 27-node scatter of one CTA's particles (P2G and the G2P adjoint), without atomics on
// the chunk's own overlaps.  Both scatters have the form
//     value(node base + o) = W_o (q + (o_x - 1) c0 + (o_y - 1) c1 + (o_z - 1) c2),  W_o = wx[o_x] wy[o_y] wz[o_z],
// q the affine part at the middle node of the stencil (expanding about it keeps the offsets in
// {-1, 0, 1} and the cancellation between q and the c terms small when the c terms dominate, as the
// stress does for stiff materials).
// The CTA's consecutive particles (spatially sorted) are reduced to the bounding box of their base
// cells.  If the box holds at most TILE_MAX nodes and one environment, every particle writes its
// stencil record (base, 9 weights, q, c0, c1, c2) to shared memory and each thread owns nodes of
// the box: it sums the contributions of the chunk's particles whose stencil covers its node and
// issues one 16-byte vector RED per node — the CTA's same-node contributions never meet in an
// atomic.  Otherwise (dispersed particles) each particle issues its 27 vector REDs directly.
// `mark_box` is called for the box when it is compact, `mark_one` per particle otherwise.
// Shared memory: 25 * NT words.
struct StencilRec {
  float wx[3], wy[3], wz[3];
  float4 q;
  v3 c0, c1, c2;
};

// MODE: DT_SCATTER_TILE, DT_SCATTER_GLOBAL, or DT_SCATTER_WARP + d for the warp reduction capped at
// d shuffle steps (d = 0: whole runs; dt_world.scatter_depth selects d at launch).  MARK: the scatter
// marks the grid blocks it touches (P2G); without it (the G2P adjoint) the warp and global modes need
// no bounding box and skip its two CTA barriers.
template <int NT, int TILE_MAX, int MODE, bool MARK = true, typename MarkBox, typename MarkOne>
DT_DEV void stencil_scatter(const dt_world& w, int chunk, bool ok, int env, const int base[3], const StencilRec& r,
                            float* sm, int* sh, float4* dst, const MarkBox& mark_box, const MarkOne& mark_one) {
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  // the CTA's box of base cells: for the tile modes, and for marking in the global mode; the warp mode
  // marks per warp (below), without CTA barriers
  constexpr bool BOX = MODE == DT_SCATTER_TILE || MODE >= DT_MODE_SMEM || (MARK && MODE == DT_SCATTER_GLOBAL);
  int L0 = 0, L1 = 0, L2 = 0, ex = 0, ey = 0, ez = 0, tile_n = 0;
  bool compact = false;
  if constexpr (BOX) {
    if (tid == 0) {
      sh[0] = sh[1] = sh[2] = 0x7fffffff;
      sh[3] = sh[4] = sh[5] = (int)0x80000000;
      const int p0 = chunk * NT, p1 = min(p0 + NT, w.n_particles) - 1;
      sh[6] = (w.p_env[p0] == w.p_env[p1]) ? 1 : 0;
    }
    __syncthreads();
    int lo0 = ok ? base[0] : 0x7fffffff, lo1 = ok ? base[1] : 0x7fffffff, lo2 = ok ? base[2] : 0x7fffffff;
    int hi0 = ok ? base[0] : (int)0x80000000, hi1 = ok ? base[1] : (int)0x80000000,
        hi2 = ok ? base[2] : (int)0x80000000;
    lo0 = __reduce_min_sync(0xffffffffu, lo0);
    lo1 = __reduce_min_sync(0xffffffffu, lo1);
    lo2 = __reduce_min_sync(0xffffffffu, lo2);
    hi0 = __reduce_max_sync(0xffffffffu, hi0);
    hi1 = __reduce_max_sync(0xffffffffu, hi1);
    hi2 = __reduce_max_sync(0xffffffffu, hi2);
    if (lane == 0 && hi0 != (int)0x80000000) {
      atomicMin(sh + 0, lo0);
      atomicMin(sh + 1, lo1);
      atomicMin(sh + 2, lo2);
      atomicMax(sh + 3, hi0);
      atomicMax(sh + 4, hi1);
      atomicMax(sh + 5, hi2);
    }
    __syncthreads();
    L0 = sh[0];
    L1 = sh[1];
    L2 = sh[2];
    const bool any = sh[3] != (int)0x80000000;
    ex = any ? sh[3] - L0 + 3 : 0;
    ey = any ? sh[4] - L1 + 3 : 0;
    ez = any ? sh[5] - L2 + 3 : 0;
    tile_n = ex * ey * ez;
    compact = any && sh[6] && tile_n <= TILE_MAX;
    if (compact) {
      const dt_env& E0 = w.envs[w.p_env[min(chunk * NT, w.n_particles - 1)]];
      mark_box(E0, L0, L1, L2, L0 + ex - 1, L1 + ey - 1, L2 + ez - 1, tid, NT);
    }
  }  // BOX
  const bool gather = MODE == DT_SCATTER_TILE && compact;
  if (gather) {
    // stencil records, structure of arrays: rows 0-2 base (int bits), 3-11 weights, 12-15 q, 16-24 c
    float* rec = sm;
    rec[0 * NT + tid] = __int_as_float(ok ? base[0] - L0 : -1000);
    rec[1 * NT + tid] = __int_as_float(ok ? base[1] - L1 : -1000);
    rec[2 * NT + tid] = __int_as_float(ok ? base[2] - L2 : -1000);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      rec[(3 + i) * NT + tid] = r.wx[i];
      rec[(6 + i) * NT + tid] = r.wy[i];
      rec[(9 + i) * NT + tid] = r.wz[i];
    }
    rec[12 * NT + tid] = r.q.x;
    rec[13 * NT + tid] = r.q.y;
    rec[14 * NT + tid] = r.q.z;
    rec[15 * NT + tid] = r.q.w;
    rec[16 * NT + tid] = r.c0.x;
    rec[17 * NT + tid] = r.c0.y;
    rec[18 * NT + tid] = r.c0.z;
    rec[19 * NT + tid] = r.c1.x;
    rec[20 * NT + tid] = r.c1.y;
    rec[21 * NT + tid] = r.c1.z;
    rec[22 * NT + tid] = r.c2.x;
    rec[23 * NT + tid] = r.c2.y;
    rec[24 * NT + tid] = r.c2.z;
    __syncthreads();
    const int cnt = min(NT, w.n_particles - chunk * NT);
    const dt_env& E0 = w.envs[w.p_env[min(chunk * NT, w.n_particles - 1)]];
    const int node_off = E0.node_off, nb1 = E0.nb[1], nb2 = E0.nb[2];
    for (int n = tid; n < tile_n; n += NT) {
      const int nc = n % ez, nbb = (n / ez) % ey, na = n / (ey * ez);
      float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
      for (int p = 0; p < cnt; ++p) {
        const int oi = na - __float_as_int(rec[p]);
        const int oj = nbb - __float_as_int(rec[NT + p]);
        const int ok_ = nc - __float_as_int(rec[2 * NT + p]);
        if ((unsigned)oi <= 2u && (unsigned)oj <= 2u && (unsigned)ok_ <= 2u) {
          const float W = (rec[(3 + oi) * NT + p] * rec[(6 + oj) * NT + p]) * rec[(9 + ok_) * NT + p];
          const float fi = (float)(oi - 1), fj = (float)(oj - 1), fk = (float)(ok_ - 1);
          ax += W * (((rec[12 * NT + p] + fi * rec[16 * NT + p]) + fj * rec[19 * NT + p]) + fk * rec[22 * NT + p]);
          ay += W * (((rec[13 * NT + p] + fi * rec[17 * NT + p]) + fj * rec[20 * NT + p]) + fk * rec[23 * NT + p]);
          az += W * (((rec[14 * NT + p] + fi * rec[18 * NT + p]) + fj * rec[21 * NT + p]) + fk * rec[24 * NT + p]);
          aw += W * rec[15 * NT + p];
        }
      }
      if (aw != 0.f || ax != 0.f || ay != 0.f || az != 0.f) {
        const int i = L0 + na, j = L1 + nbb, k = L2 + nc;
        const int g = node_off + ((((i >> 2) * nb1 + (j >> 2)) * nb2 + (k >> 2)) << 6) + ((i & 3) << 4) +
                      ((j & 3) << 2) + (k & 3);
        red_add_v4(dst + g, make_float4(ax, ay, az, aw));
      }
    }
  } else if constexpr (MODE >= DT_SCATTER_WARP) {
    // segmented reduction over runs of lanes with the same base node (same env and cell): every
    // lane of the warp takes part in the shuffles; lanes without a particle form runs of their own.
    // SMEM: the run sums go into a shared-memory tile of the CTA's box of nodes (shared atomics),
    // flushed with one vector RED per touched node once every warp has added
    constexpr bool SMEM = MODE >= DT_MODE_SMEM;
    const bool in_tile = SMEM && compact && tile_n <= DT_SMEM_TILE;  // CTA-uniform
    if (in_tile) {
      for (int n = tid; n < 4 * tile_n; n += NT) sm[n] = 0.f;
      __syncthreads();
    }
    int node_off = 0, nb1 = 1, nb2 = 1;
    if (ok) {
      const dt_env& E = w.envs[env];
      node_off = E.node_off;
      nb1 = E.nb[1];
      nb2 = E.nb[2];
    }
    const StencilNodes sn = stencil_nodes(node_off, nb1, nb2, base);
    const int key = ok ? sn.x[0] + sn.y[0] + sn.z[0] : -1 - lane;
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    const bool head = lane == 0 || prev != key;
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const unsigned after = lane == 31 ? 0u : (heads >> (lane + 1)) << (lane + 1);
    const int seg_end = after ? __ffs(after) - 1 : 32;
    const int run = __reduce_max_sync(0xffffffffu, head ? seg_end - lane : 0);
    int steps = run > 1 ? 32 - __clz(run - 1) : 0;
    // MODE = DT_SCATTER_WARP + depth (or DT_MODE_SMEM + depth): at most `depth` shuffle steps (0: the
    // whole run)
    constexpr int DEPTH = SMEM ? MODE - DT_MODE_SMEM : MODE - DT_SCATTER_WARP;
    if constexpr (DEPTH > 0) steps = min(steps, DEPTH);
    // after `steps` steps a lane holds the sum of its window of 2^steps lanes (clipped to the run);
    // the first lane of every window issues the RED
    const int seg_start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
    const bool issuer = ((lane - seg_start) & ((1 << steps) - 1)) == 0;
#pragma unroll
    for (int oi = 0; oi < 3; ++oi)
#pragma unroll
      for (int oj = 0; oj < 3; ++oj)
#pragma unroll
        for (int ok_ = 0; ok_ < 3; ++ok_) {
          const float W = ok ? (r.wx[oi] * r.wy[oj]) * r.wz[ok_] : 0.f;
          const float fi = (float)(oi - 1), fj = (float)(oj - 1), fk = (float)(ok_ - 1);
          const v3 t = ((v3{r.q.x, r.q.y, r.q.z} + fi * r.c0) + fj * r.c1) + fk * r.c2;
          float4 a = make_float4(W * t.x, W * t.y, W * t.z, W * r.q.w);
          for (int s = 0; s < steps; ++s) {
            const int off = 1 << s;
            const float bx = __shfl_down_sync(0xffffffffu, a.x, off);
            const float by = __shfl_down_sync(0xffffffffu, a.y, off);
            const float bz = __shfl_down_sync(0xffffffffu, a.z, off);
            const float bw = __shfl_down_sync(0xffffffffu, a.w, off);
            if (lane + off < seg_end) {
              a.x += bx;
              a.y += by;
              a.z += bz;
              a.w += bw;
            }
          }
          if (issuer && ok) {
            if (in_tile) {
              float* t = sm + 4 * (((base[0] - L0 + oi) * ey + (base[1] - L1 + oj)) * ez + (base[2] - L2 + ok_));
              atomicAdd(t + 0, a.x);
              atomicAdd(t + 1, a.y);
              atomicAdd(t + 2, a.z);
              if (a.w != 0.f) atomicAdd(t + 3, a.w);
            } else {
              red_add_v4(dst + ((sn.x[oi] + sn.y[oj]) + sn.z[ok_]), a);
            }
          }
        }
    if (in_tile) {
      __syncthreads();
      const dt_env& E0 = w.envs[w.p_env[min(chunk * NT, w.n_particles - 1)]];
      const int t_off = E0.node_off, t_nb1 = E0.nb[1], t_nb2 = E0.nb[2];
      const float4* tl = reinterpret_cast<const float4*>(sm);
      for (int n = tid; n < tile_n; n += NT) {
        const float4 v = tl[n];
        if (v.x == 0.f && v.y == 0.f && v.z == 0.f && v.w == 0.f) continue;
        const int nc = n % ez, nbb = (n / ez) % ey, na = n / (ey * ez);
        const int i = L0 + na, j = L1 + nbb, k = L2 + nc;
        const int g = t_off + ((((i >> 2) * t_nb1 + (j >> 2)) * t_nb2 + (k >> 2)) << 6) + ((i & 3) << 4) +
                      ((j & 3) << 2) + (k & 3);
        red_add_v4(dst + g, v);
      }
    }
    if constexpr (MARK && !SMEM) {
      // the blocks this warp's stencils touch: the warp's box of base cells (+2 nodes) when its
      // particles share one environment and the box spans at most 32 blocks, else per particle
      const int e_lo = __reduce_min_sync(0xffffffffu, ok ? env : 0x7fffffff);
      const int e_hi = __reduce_max_sync(0xffffffffu, ok ? env : -1);
      if (e_hi >= 0) {  // warp-uniform: some particle of the warp was scattered
        const int l0 = __reduce_min_sync(0xffffffffu, ok ? base[0] : 0x7fffffff);
        const int l1 = __reduce_min_sync(0xffffffffu, ok ? base[1] : 0x7fffffff);
        const int l2 = __reduce_min_sync(0xffffffffu, ok ? base[2] : 0x7fffffff);
        const int h0 = __reduce_max_sync(0xffffffffu, ok ? base[0] + 2 : -1);
        const int h1 = __reduce_max_sync(0xffffffffu, ok ? base[1] + 2 : -1);
        const int h2 = __reduce_max_sync(0xffffffffu, ok ? base[2] + 2 : -1);
        const int nbx = (h0 >> 2) - (l0 >> 2) + 1, nby = (h1 >> 2) - (l1 >> 2) + 1, nbz = (h2 >> 2) - (l2 >> 2) + 1;
        if (e_lo == e_hi && nbx * nby * nbz <= 32) {
          mark_box(w.envs[e_lo], l0, l1, l2, h0, h1, h2, lane, 32);
        } else if (ok) {
          mark_one(w.envs[env]);
        }
      }
    } else if (MARK && ok && !compact) {
      mark_one(w.envs[env]);
    }
  } else if (ok) {
    const dt_env& E = w.envs[env];
    const StencilNodes sn = stencil_nodes(E, base);
#pragma unroll
    for (int oi = 0; oi < 3; ++oi)
#pragma unroll
      for (int oj = 0; oj < 3; ++oj)
#pragma unroll
        for (int ok_ = 0; ok_ < 3; ++ok_) {
          const int n = (sn.x[oi] + sn.y[oj]) + sn.z[ok_];
          const float W = (r.wx[oi] * r.wy[oj]) * r.wz[ok_];
          const float fi = (float)(oi - 1), fj = (float)(oj - 1), fk = (float)(ok_ - 1);
          const v3 t = ((v3{r.q.x, r.q.y, r.q.z} + fi * r.c0) + fj * r.c1) + fk * r.c2;
          red_add_v4(dst + n, make_float4(W * t.x, W * t.y, W * t.z, W * r.q.w));
        }
    if (!compact) mark_one(E);
  }
}

// bit-reproducible centroid distance (find_closest, fem_sensor.py:352-353): every operation
// separately rounded so that the argmin matches the CPU restatement exactly
DT_DEV float cent_dist(float4 c, float px, float py, float pz) {
  float dx = __fsub_rn(c.x, px), dy = __fsub_rn(c.y, py), dz = __fsub_rn(c.z, pz);
  float s = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  return __fsqrt_rn(__fadd_rn(s, 1e-10f));
}
