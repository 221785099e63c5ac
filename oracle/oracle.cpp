// ORACLE — test infrastructure only.  CPU restatement of the DiffTactile simulation substep
// (Taichi kernels of the reference), used as the parity oracle of the CUDA path and as the
// timed CPU baseline.  It is never linked into or called by the product path.
//
// Parity status: the forward substep is pinned against the reference's own simulation methods.
// The reference is Taichi 1.6.0 code (un-vendored third-party JIT, not importable in this image)
// and ships no tests, golden vectors or fixtures for this path; tests/golden/make_substep.py runs
// its MPMObj (mpm_elastic.py, mpm_plastic.py), FEMDomeSensor (fem_sensor.py) and Contact.update
// (grasp_plastic.py) methods, read from the reference source, in float64 on a numpy stand-in for
// the Taichi primitives, and tests/test_golden_substep.py finds this restatement within 2e-15 of
// them (particles, grid, contact argmin, sensor forces and next frame; the rope and the gripper's
// update2 through the cable task's Contact.update).  The adjoints (Taichi autodiff in the
// reference) are checked against central differences of the reference's own substep
// (tests/golden/make_gradient.py, tests/test_golden_gradient.py), against the reference's
// hand-written SVD adjoint (tests/test_golden_svdgrad.py), by analytic known-answer tests and by
// central differences of this restatement in double precision.
//
// Structure follows the reference kernel by kernel, on a dense per-frame grid in (i, j, k)
// row-major order exactly like the Taichi fields, processing particles/nodes/tets in index
// order:
//   compute_new_F   difftactile/object_model/mpm_elastic.py:135-137
//   svd             difftactile/object_model/mpm_elastic.py:140-142 (ti.svd; restated below as
//                   cyclic Jacobi on A^T A + column sort + Givens QR, see svd3)
//   p2g             difftactile/object_model/mpm_elastic.py:176-208,
//                   difftactile/object_model/mpm_plastic.py:222-256 (von Mises :151-166),
//                   difftactile/object_model/multi_obj.py:228-252 (per-particle material)
//   check_grid_occupy  difftactile/object_model/mpm_elastic.py:211-214
//   check_collision difftactile/tasks/grasp_plastic.py:270-276 + find_closest
//                   difftactile/sensor_model/fem_sensor.py:344-359
//   collision       difftactile/tasks/grasp_plastic.py:280-299 + find_sdf fem_sensor.py:362-394
//                   + calculate_contact_force grasp_plastic.py:205-216
//                   + update_contact_force mpm_elastic.py:131-132, fem_sensor.py:402-406
//   grid_op         difftactile/object_model/mpm_elastic.py:217-240
//   g2p             difftactile/object_model/mpm_elastic.py:244-260
//   FEM update      difftactile/sensor_model/fem_sensor.py:409-440 (= gripper_fem.py:375-401)
//   FEM update2     difftactile/sensor_model/fem_sensor.py:444-457, gripper_fem.py:404-418
//   order           Contact.update, difftactile/tasks/grasp_plastic.py:151-164
//
// Build: oracle/build.py (g++ -O2 -ffp-contract=off -fopenmp -shared).  -ffp-contract=off keeps
// every float operation separately rounded, so the argmin of find_closest is bit-reproducible.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

typedef struct orc_sensor {
  int nv, nt, nf;
  const int* tets;    // [nt][4] local vertex ids
  const int* tris;    // [nf][3] local vertex ids
  const int* layer;   // [nv]
  const double* B;    // [nt][9] rest-shape inverse (row-major)
  double mass, mu, lam;
  double out_dir[3];
  int carry;          // 1: gripper_fem.py:415 velocity carry term
  int model;          // 0: the reference's elastomer force (fem_sensor.py:424-435), 1: linear corotated
} orc_sensor;

// PBD rope (PBD_rope.py) with its sensor contact parameters (cable_straightening.py:212-224)
typedef struct orc_rope {
  int n;              // particles; node 0 is pinned at pin
  int iters;          // repetitions of the stretch + bending pass pair (<= 1: one, as PBD_rope.py:132-172)
  double mass, rad;   // p_mass = rho 4/3 pi rad^3, contact offset = rad
  double rest, bend;  // rest_length, bending_length
  double alpha_s, alpha_b;    // compliance / dt^2
  double relax_s, relax_b;    // stretch_relaxation, bending_relaxation
  double table_h, friction;   // floor height and tangential velocity factor
  double grav[3], pin[3];
  double kn, kd, kt, mu_t;
} orc_rope;

// per-rope arrays of one substep (element type float or double as the entry point)
typedef struct orc_rope_io {
  void* pos;          // [n][3] frame f
  void* vel;          // [n][3]
  void* trav;         // [n] travel_info
  void* pos1;         // [n][3] frame f+1 (written)
  void* vel1;
  void* trav1;
  void* ext;          // [n][3] ext_f[f]: sum of contact force * dt (written)
  int* cidx;          // [n][n_sensors] argmin per sensor (written)
  const void* posb1;  // adjoints of frame f+1 (backward)
  const void* velb1;
  const void* travb1;
  void* posb;         // adjoints of frame f (written by the backward)
  void* velb;
  void* travb;
} orc_rope_io;

typedef struct orc_scene {
  int n_particles;
  int n[3];
  int bound, bc;
  double dx, inv_dx, p_vol, p_mass, dt, eps;
  double grav[3];
  double kn, kd, kt, mu_t;
  int n_materials;
  int n_sensors;
  const double* mat_mu;
  const double* mat_lam;
  const double* mat_yield;
  const int* mat_model;
  const int* p_mat;   // [n_particles]
  const orc_sensor* sensors;
  int svd_sweeps;
  int n_threads;      // OpenMP threads for the timed baseline (<=1: sequential)
  double grad_clip;   // backward clamp (grasp_plastic.py:192-202); 0 disables
  int n_ropes;
  int pad2_;
  const orc_rope* ropes;
  orc_rope_io* rope_io;  // [n_ropes]
  // optional [n_particles] branch of the von Mises return map: -1 decided by the yield test, 0 elastic,
  // 1 yielding (a comparison pins the branch another implementation took for particles on the yield
  // surface, where the test's outcome depends on rounding); NULL: every particle decided by the test
  const signed char* yield_branch;
} orc_scene;

}  // extern "C"

namespace {

enum { MODEL_COROTATED = 0, MODEL_VON_MISES = 1, MODEL_NEOHOOKEAN = 2 };

template <typename T>
struct M3 {
  T a[3][3];
};

template <typename T>
inline M3<T> mzero() {
  M3<T> m;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m.a[i][j] = T(0);
  return m;
}
template <typename T>
inline M3<T> meye() {
  M3<T> m = mzero<T>();
  m.a[0][0] = m.a[1][1] = m.a[2][2] = T(1);
  return m;
}
template <typename T>
inline M3<T> mmul(const M3<T>& x, const M3<T>& y) {
  M3<T> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T s = x.a[i][0] * y.a[0][j];
      s = s + x.a[i][1] * y.a[1][j];
      s = s + x.a[i][2] * y.a[2][j];
      r.a[i][j] = s;
    }
  return r;
}
template <typename T>
inline M3<T> mT(const M3<T>& x) {
  M3<T> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[j][i];
  return r;
}
template <typename T>
inline T mdet(const M3<T>& m) {
  const T(*a)[3] = m.a;
  return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
         a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}
// cofactor matrix: cof[i][j] = d det / d a[i][j]
template <typename T>
inline M3<T> mcof(const M3<T>& m) {
  const T(*a)[3] = m.a;
  M3<T> c;
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

// ---------------------------------------------------------------------------------------------
// 3x3 SVD with the convention of ti.svd: A = U diag(s) V^T, det U = det V = +1, |s0|>=|s1|>=|s2|,
// s0, s1 >= 0 and s2 carrying the sign of det A.
// Method (published, restated): cyclic Jacobi eigen-decomposition of A^T A with the classical
// rotation of Golub & Van Loan, "Matrix Computations", Alg. 8.4.1 (sym.schur2); columns of
// B = A V sorted by norm with a sign flip per swap to keep det V = +1; Givens QR of B for U and
// the signed singular values — the outline of McAdams et al. 2011, "Computing the SVD of 3x3
// matrices with minimal branching and elementary floating point operations", with exact rather
// than approximate rotation angles.
template <typename T>
inline void jacobi_rot(T S[3][3], T V[3][3], int p, int q) {
  T apq = S[p][q];
  if (apq == T(0)) return;
  T tau = (S[q][q] - S[p][p]) / (T(2) * apq);
  T t = (tau >= T(0) ? T(1) : T(-1)) / (std::fabs(tau) + std::sqrt(T(1) + tau * tau));
  T c = T(1) / std::sqrt(T(1) + t * t);
  T s = t * c;
  for (int k = 0; k < 3; ++k) {  // S <- S J
    T sp = S[k][p], sq = S[k][q];
    S[k][p] = c * sp - s * sq;
    S[k][q] = s * sp + c * sq;
  }
  for (int k = 0; k < 3; ++k) {  // S <- J^T S
    T sp = S[p][k], sq = S[q][k];
    S[p][k] = c * sp - s * sq;
    S[q][k] = s * sp + c * sq;
  }
  for (int k = 0; k < 3; ++k) {  // V <- V J
    T vp = V[k][p], vq = V[k][q];
    V[k][p] = c * vp - s * vq;
    V[k][q] = s * vp + c * vq;
  }
}

template <typename T>
inline void swap_cols_neg(T B[3][3], T V[3][3], int i, int j) {
  for (int k = 0; k < 3; ++k) {
    T b = B[k][i];
    B[k][i] = B[k][j];
    B[k][j] = -b;
    T v = V[k][i];
    V[k][i] = V[k][j];
    V[k][j] = -v;
  }
}

template <typename T>
inline void qr_givens(T B[3][3], T U[3][3], int i, int j, int col) {
  // zero B[j][col] by rotating rows i and j
  T a = B[i][col], b = B[j][col];
  T r = std::sqrt(a * a + b * b);
  T c = T(1), s = T(0);
  if (r > T(1e-30)) {
    c = a / r;
    s = b / r;
  }
  for (int k = 0; k < 3; ++k) {
    T bi = B[i][k], bj = B[j][k];
    B[i][k] = c * bi + s * bj;
    B[j][k] = -s * bi + c * bj;
  }
  for (int k = 0; k < 3; ++k) {  // U <- U G^T
    T ui = U[k][i], uj = U[k][j];
    U[k][i] = c * ui + s * uj;
    U[k][j] = -s * ui + c * uj;
  }
}

template <typename T>
void svd3(const M3<T>& A, M3<T>& U, T s[3], M3<T>& V, int sweeps) {
  T S[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T acc = A.a[0][i] * A.a[0][j];
      acc = acc + A.a[1][i] * A.a[1][j];
      acc = acc + A.a[2][i] * A.a[2][j];
      S[i][j] = acc;
    }
  T Vm[3][3] = {{T(1), T(0), T(0)}, {T(0), T(1), T(0)}, {T(0), T(0), T(1)}};
  for (int it = 0; it < sweeps; ++it) {
    jacobi_rot(S, Vm, 0, 1);
    jacobi_rot(S, Vm, 0, 2);
    jacobi_rot(S, Vm, 1, 2);
  }
  T B[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T acc = A.a[i][0] * Vm[0][j];
      acc = acc + A.a[i][1] * Vm[1][j];
      acc = acc + A.a[i][2] * Vm[2][j];
      B[i][j] = acc;
    }
  auto cn = [&](int j) {
    T r = B[0][j] * B[0][j];
    r = r + B[1][j] * B[1][j];
    r = r + B[2][j] * B[2][j];
    return r;
  };
  if (cn(0) < cn(1)) swap_cols_neg(B, Vm, 0, 1);
  if (cn(0) < cn(2)) swap_cols_neg(B, Vm, 0, 2);
  if (cn(1) < cn(2)) swap_cols_neg(B, Vm, 1, 2);
  T Um[3][3] = {{T(1), T(0), T(0)}, {T(0), T(1), T(0)}, {T(0), T(0), T(1)}};
  qr_givens(B, Um, 0, 1, 0);
  qr_givens(B, Um, 0, 2, 0);
  qr_givens(B, Um, 1, 2, 1);
  s[0] = B[0][0];
  s[1] = B[1][1];
  s[2] = B[2][2];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      U.a[i][j] = Um[i][j];
      V.a[i][j] = Vm[i][j];
    }
}

// quadratic B-spline weights (mpm_elastic.py:181) and their derivatives
template <typename T>
inline void bspline(T fx, T w[3], T dw[3]) {
  T a = T(1.5) - fx, b = fx - T(1), c = fx - T(0.5);
  w[0] = T(0.5) * (a * a);
  w[1] = T(0.75) - b * b;
  w[2] = T(0.5) * (c * c);
  dw[0] = fx - T(1.5);
  dw[1] = T(-2) * b;
  dw[2] = c;
}

template <typename T>
struct Consts {
  T dx, inv_dx, p_mass, stress_k, eps, g2p_k, dt;
  T dt_g[3];
  T kn, kd, kt, mu_t;
  T third;
  bool clamp_vn;  // grasp variant max(v_n, 0); the cable variant (cable_straightening.py:212-224) has none
};

template <typename T>
Consts<T> make_consts(const orc_scene* sc) {
  Consts<T> k;
  k.dx = T(sc->dx);
  k.inv_dx = T(sc->inv_dx);
  k.p_mass = T(sc->p_mass);
  k.stress_k = T(-sc->dt * sc->p_vol * 4.0 * sc->inv_dx * sc->inv_dx);
  k.eps = T(sc->eps);
  k.g2p_k = T(4.0 * sc->inv_dx);
  k.dt = T(sc->dt);
  for (int d = 0; d < 3; ++d) k.dt_g[d] = T(sc->dt * sc->grav[d]);
  k.kn = T(sc->kn);
  k.kd = T(sc->kd);
  k.kt = T(sc->kt);
  k.mu_t = T(sc->mu_t);
  k.third = T(1.0 / 3.0);
  k.clamp_vn = true;
  return k;
}

inline size_t gidx(const int* n, int i, int j, int k) { return (size_t(i) * n[1] + j) * n[2] + k; }

// von Mises return mapping, mpm_plastic.py:151-166.  Returns F unchanged when not yielding.
template <typename T>
M3<T> von_mises(const M3<T>& F, const M3<T>& U, const T sig[3], const M3<T>& V, T mu, T yield_stress,
                bool* yielded = nullptr, int branch = -1) {
  T eps[3];
  for (int d = 0; d < 3; ++d) eps[d] = std::log(std::max(sig[d], T(0.05)));
  T mean = ((eps[0] + eps[1]) + eps[2]) / T(3);
  T eh[3] = {eps[0] - mean, eps[1] - mean, eps[2] - mean};
  T nrm = std::sqrt(((eh[0] * eh[0] + eh[1] * eh[1]) + eh[2] * eh[2]) + T(1e-8));
  T dg = nrm - yield_stress / (T(2) * mu);
  const bool yield = branch < 0 ? dg > T(0) : branch == 1;
  if (yielded) *yielded = yield;
  if (yield) {
    T e[3];
    for (int d = 0; d < 3; ++d) e[d] = std::exp(eps[d] - (dg / nrm) * eh[d]);
    M3<T> r;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        T acc = U.a[i][0] * e[0] * V.a[j][0];
        acc = acc + U.a[i][1] * e[1] * V.a[j][1];
        acc = acc + U.a[i][2] * e[2] * V.a[j][2];
        r.a[i][j] = acc;
      }
    return r;
  }
  return F;
}

template <typename T>
inline void cross(const T a[3], const T b[3], T r[3]) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
template <typename T>
inline T dot3(const T a[3], const T b[3]) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

// find_closest, fem_sensor.py:344-359: argmin of centroid distance, strict '<', start 100.
template <typename T>
int find_closest(const orc_sensor& s, const T* pos, const T p[3]) {
  T best = T(100.0);
  int bi = -1;
  const T third = T(1.0 / 3.0);
  for (int k = 0; k < s.nf; ++k) {
    const int* t = s.tris + 3 * k;
    T d[3];
    for (int c = 0; c < 3; ++c) {
      T pc = third * ((pos[3 * t[0] + c] + pos[3 * t[1] + c]) + pos[3 * t[2] + c]);
      d[c] = pc - p[c];
    }
    T off = std::sqrt(((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + T(1e-10));
    if (off < best) {
      best = off;
      bi = k;
    }
  }
  return bi;
}

template <typename T>
struct SdfOut {
  T sdf, nrm[3], rel[3];
  bool flag;
};

// find_sdf, fem_sensor.py:362-394.  Returns the normal already flipped (= -norm_v) and the
// relative velocity already negated (= -relative_v), as passed to calculate_contact_force.
template <typename T>
SdfOut<T> find_sdf(const orc_sensor& s, const T* pos, const T* vel, int k, const T p[3], const T gv[3],
                   T offset = T(0)) {
  const int* t = s.tris + 3 * k;
  const T* p1 = pos + 3 * t[0];
  const T* p2 = pos + 3 * t[1];
  const T* p3 = pos + 3 * t[2];
  T e1[3], e2[3], n[3];
  for (int c = 0; c < 3; ++c) {
    e1[c] = p2[c] - p1[c];
    e2[c] = p3[c] - p1[c];
  }
  cross(e1, e2, n);
  T len = std::sqrt(dot3(n, n));
  T inv = T(1) / (len + T(1e-10));
  for (int c = 0; c < 3; ++c) n[c] = inv * n[c];
  T od[3] = {T(s.out_dir[0]), T(s.out_dir[1]), T(s.out_dir[2])};
  T sg = dot3(n, od) < T(0) ? T(-1) : T(1);
  for (int c = 0; c < 3; ++c) n[c] = sg * n[c];
  T ds[3] = {p[0] - p1[0], p[1] - p1[1], p[2] - p1[2]};
  T sdf = dot3(ds, n);
  T proj[3];
  for (int c = 0; c < 3; ++c) proj[c] = p[c] - sdf * n[c];
  T v0[3], v1[3], v2[3];
  for (int c = 0; c < 3; ++c) {
    v0[c] = p3[c] - p1[c];
    v1[c] = p2[c] - p1[c];
    v2[c] = proj[c] - p1[c];
  }
  T d00 = dot3(v0, v0), d01 = dot3(v0, v1), d02 = dot3(v0, v2), d11 = dot3(v1, v1), d12 = dot3(v1, v2);
  T invd = T(1) / (d00 * d11 - d01 * d01);
  T u = (d11 * d02 - d01 * d12) * invd;
  T v = (d00 * d12 - d01 * d02) * invd;
  SdfOut<T> o;
  sdf -= offset;  // PBD collision offset (fem_sensor.py:388), after the projection
  o.sdf = sdf;
  const T third = T(1.0 / 3.0);
  for (int c = 0; c < 3; ++c) {
    o.nrm[c] = n[c];
    T tv = third * ((vel[3 * t[0] + c] + vel[3 * t[1] + c]) + vel[3 * t[2] + c]);
    o.rel[c] = -(gv[c] - tv);
  }
  o.flag = sdf < T(0) && u >= T(0) && v >= T(0) && (u + v <= T(1));
  return o;
}

// calculate_contact_force, grasp_plastic.py:205-216, called with (sdf, n, r) = (sdf, -norm_v, -rel_v)
template <typename T>
void contact_force(const Consts<T>& K, T sdf, const T n[3], const T r[3], T ext[3]) {
  T nr = dot3(n, r);
  T vn = K.clamp_vn ? std::max(nr, T(0)) : nr;
  T fn[3];
  T kk = K.kn + K.kd * vn;
  for (int c = 0; c < 3; ++c) fn[c] = -kk * sdf * n[c];
  T vt[3];
  for (int c = 0; c < 3; ++c) vt[c] = r[c] - nr * n[c];
  T vtn = std::sqrt(dot3(vt, vt) + T(1e-11));
  T ft[3] = {T(0), T(0), T(0)};
  if (vtn > T(1e-4)) {
    T fnn = std::sqrt(dot3(fn, fn));
    T g = std::min(K.kt * vtn, K.mu_t * fnn);
    for (int c = 0; c < 3; ++c) ft[c] = (vt[c] / vtn) * g;
  }
  for (int c = 0; c < 3; ++c) ext[c] = fn[c] + ft[c];
}

template <typename T>
struct Particle {
  M3<T> C, F;
  T x[3], v[3];
};

template <typename T>
inline Particle<T> load_particle(const T* x, const T* v, const T* C, const T* F, int p) {
  Particle<T> q;
  for (int d = 0; d < 3; ++d) {
    q.x[d] = x[3 * p + d];
    q.v[d] = v[3 * p + d];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      q.C.a[i][j] = C[9 * p + 3 * i + j];
      q.F.a[i][j] = F[9 * p + 3 * i + j];
    }
  return q;
}

// Per-particle forward quantities shared by p2g and its adjoint.
template <typename T>
struct P2GFwd {
  int base[3];
  T fx[3], w[3][3], dw[3][3];
  M3<T> Fn, U, V, Fp, R, affine, cauchy;
  T sig[3], J;
  int model;
  bool yield;
  T mu, lam, ys;
};

template <typename T>
bool particle_base(const orc_scene* sc, const Consts<T>& K, const T x[3], int base[3], T fx[3]) {
  bool ok = true;
  for (int d = 0; d < 3; ++d) {
    T g = x[d] * K.inv_dx - T(0.5);
    base[d] = int(g);  // truncation toward zero, like Taichi's cast(int)
    fx[d] = x[d] * K.inv_dx - T(base[d]);
    if (!(g == g) || base[d] < 0 || base[d] + 2 >= sc->n[d]) ok = false;
  }
  return ok;
}

template <typename T>
void p2g_particle(const orc_scene* sc, const Consts<T>& K, const Particle<T>& q, int p, P2GFwd<T>& o) {
  for (int d = 0; d < 3; ++d) {
    T wd[3], dwd[3];
    bspline(o.fx[d], wd, dwd);
    for (int i = 0; i < 3; ++i) {
      o.w[i][d] = wd[i];
      o.dw[i][d] = dwd[i];
    }
  }
  // compute_new_F: (I + dt C) F
  M3<T> A = meye<T>();
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A.a[i][j] = A.a[i][j] + K.dt * q.C.a[i][j];
  o.Fn = mmul(A, q.F);
  svd3(o.Fn, o.U, o.sig, o.V, sc->svd_sweeps);
  int m = sc->p_mat ? sc->p_mat[p] : 0;
  o.mu = T(sc->mat_mu[m]);
  o.lam = T(sc->mat_lam[m]);
  o.ys = T(sc->mat_yield[m]);
  o.model = sc->mat_model[m];
  o.yield = false;
  o.R = mmul(o.U, mT(o.V));
  if (o.model == MODEL_VON_MISES) {
    o.Fp = von_mises(o.Fn, o.U, o.sig, o.V, o.mu, o.ys, &o.yield, sc->yield_branch ? int(sc->yield_branch[p]) : -1);
    o.J = mdet(o.Fp);
  } else if (o.model == MODEL_NEOHOOKEAN) {
    o.Fp = o.Fn;
    o.J = mdet(o.Fp);
  } else {
    o.Fp = o.Fn;
    o.J = o.sig[0] * (o.sig[1] * o.sig[2]);
  }
  M3<T> c;
  if (o.model == MODEL_NEOHOOKEAN) {
    M3<T> FFt = mmul(o.Fp, mT(o.Fp));
    T lj = o.lam * std::log(o.J);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) c.a[i][j] = o.mu * (FFt.a[i][j] - (i == j ? T(1) : T(0))) + (i == j ? lj : T(0));
  } else {
    M3<T> D;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) D.a[i][j] = o.Fp.a[i][j] - o.R.a[i][j];
    M3<T> DFt = mmul(D, mT(o.Fp));
    T lj = o.lam * o.J * (o.J - T(1));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) c.a[i][j] = T(2) * o.mu * DFt.a[i][j] + (i == j ? lj : T(0));
  }
  o.cauchy = c;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o.affine.a[i][j] = K.stress_k * c.a[i][j] + K.p_mass * q.C.a[i][j];
}

}  // namespace

// =============================================================================================
// Forward substep, reference order of Contact.update (grasp_plastic.py:151-164).
// Sensor arrays are per sensor, [nv][3]; vel[s] is updated in place by the elastic forces
// (as the Taichi kernel does) and afterwards holds the post-force velocity used by contact.
// Dense grid outputs are [n0*n1*n2] (*3 for vectors) and are overwritten.  With n_threads > 1 the
// loops run in parallel with atomic scatters (the Taichi CPU backend's execution model); with one
// thread the summation order is the sequential index order.
// =============================================================================================
template <typename T>
inline void aadd(T& a, T b, bool atomic) {
  if (atomic) {
#pragma omp atomic
    a += b;
  } else {
    a += b;
  }
}

// ---- PBD rope: check_collision + collision (cable_straightening.py:288-319) and PBDRope.update
// (PBD_rope.py:112-180), after the sensors' elastic update and before their update2 ----
template <typename T>
Consts<T> rope_consts(const orc_scene* sc, const orc_rope& R) {
  Consts<T> K = make_consts<T>(sc);
  K.kn = T(R.kn);
  K.kd = T(R.kd);
  K.kt = T(R.kt);
  K.mu_t = T(R.mu_t);
  K.clamp_vn = false;
  return K;
}

// stretch (stride 1) or bending (stride 2) pass, Jacobi: corrections from the positions on entry
template <typename T>
void rope_pass(std::vector<T>& tp, int n, int stride, T len, T alpha, T relax, T w) {
  std::vector<T> dp(3 * n, T(0));
  for (int e = 0; e + stride < n; ++e) {
    const T* x1 = &tp[3 * e];
    const T* x2 = &tp[3 * (e + stride)];
    T d[3] = {x1[0] - x2[0], x1[1] - x2[1], x1[2] - x2[2]};
    T L = std::sqrt(dot3(d, d) + T(1e-10));
    T C = L - len;
    for (int c = 0; c < 3; ++c) {
      T dpc = -C / (w + w + alpha) * d[c] / L * relax;
      dp[3 * e + c] += dpc * w;
      dp[3 * (e + stride) + c] -= dpc * w;
    }
  }
  for (int i = 0; i < 3 * n; ++i) tp[i] += dp[i];
}

template <typename T>
void rope_integrate(const orc_rope& R, T dt, const T* rp, const T* rv, const T* re, std::vector<T>& tp,
                    std::vector<unsigned char>& floor_hit) {
  const int n = R.n;
  tp.assign(3 * n, T(0));
  floor_hit.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    T nv[3];
    for (int c = 0; c < 3; ++c) nv[c] = (rv[3 * i + c] + re[3 * i + c] / T(R.mass)) + T(R.grav[c]) * dt;
    T npy = rp[3 * i + 1] + nv[1] * dt;
    if (npy < T(R.table_h) && nv[1] < T(0)) {  // floor: drop the normal part, damp the tangential
      floor_hit[i] = 1;
      nv[1] = nv[1] - nv[1];
      nv[0] = nv[0] * T(R.friction);
      nv[1] = nv[1] * T(R.friction);
      nv[2] = nv[2] * T(R.friction);
    }
    for (int c = 0; c < 3; ++c) tp[3 * i + c] = rp[3 * i + c] + nv[c] * dt;
  }
}

template <typename T>
void rope_fwd(const orc_scene* sc, const orc_rope& R, orc_rope_io& io, T* const* pos, T* const* vel,
              T* const* ext) {
  const int n = R.n, NS = sc->n_sensors;
  const T dt = T(sc->dt);
  const Consts<T> K = rope_consts<T>(sc, R);
  const T* rp = static_cast<const T*>(io.pos);
  const T* rv = static_cast<const T*>(io.vel);
  const T* rt = static_cast<const T*>(io.trav);
  T* re = static_cast<T*>(io.ext);
  for (int p = 0; p < n; ++p) {
    bool any = false;
    for (int c = 0; c < 3; ++c) re[3 * p + c] = T(0);
    for (int s = 0; s < NS; ++s) {
      const orc_sensor& S = sc->sensors[s];
      int kk = find_closest(S, pos[s], rp + 3 * p);
      io.cidx[p * NS + s] = kk;
      if (kk < 0) continue;
      SdfOut<T> so = find_sdf(S, pos[s], vel[s], kk, rp + 3 * p, rv + 3 * p, T(R.rad));
      if (!so.flag) continue;
      T e[3];
      contact_force(K, so.sdf, so.nrm, so.rel, e);
      for (int c = 0; c < 3; ++c) re[3 * p + c] += e[c] * dt;  // update_contact_force, PBD_rope.py:104-105
      const int* t = S.tris + 3 * kk;
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) ext[s][3 * t[a] + c] += K.third * (T(-1) * e[c]);
      any = true;
    }
    static_cast<T*>(io.trav1)[p] = any ? T(1) : rt[p];
  }
  std::vector<T> tp;
  std::vector<unsigned char> fl;
  rope_integrate(R, dt, rp, rv, re, tp, fl);
  const T w = T(1) / T(R.mass);
  for (int it = 0; it < std::max(R.iters, 1); ++it) {
    rope_pass(tp, n, 1, T(R.rest), T(R.alpha_s), T(R.relax_s), w);
    rope_pass(tp, n, 2, T(R.bend), T(R.alpha_b), T(R.relax_b), w);
  }
  T* rp1 = static_cast<T*>(io.pos1);
  T* rv1 = static_cast<T*>(io.vel1);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      rp1[3 * i + c] = i == 0 ? T(R.pin[c]) : tp[3 * i + c];
      rv1[3 * i + c] = (rp1[3 * i + c] - rp[3 * i + c]) / dt;
    }
}

template <typename T>
static int substep_impl(const orc_scene* sc, const T* x, const T* v, const T* C, const T* F, T* x1, T* v1,
                        T* C1, T* F1, T* const* pos, T* const* vel, const T* const* vpos, const T* const* cv,
                        const T* const* cv1, T* const* pos1, T* const* vel1, T* const* vpos1, T* const* ext,
                        T* grid_m, T* grid_v_in, T* grid_v_out, T* grid_f, int* cidx) {
  const Consts<T> K = make_consts<T>(sc);
  const int* n = sc->n;
  const size_t nn = size_t(n[0]) * n[1] * n[2];
  const int NS = sc->n_sensors;
  const int nt = sc->n_threads > 1 ? sc->n_threads : 1;
  const bool at = nt > 1;
  int err = 0;
  std::fill(grid_m, grid_m + nn, T(0));
  std::fill(grid_v_in, grid_v_in + 3 * nn, T(0));
  std::fill(grid_v_out, grid_v_out + 3 * nn, T(0));
  std::fill(grid_f, grid_f + 3 * nn, T(0));
  for (size_t i = 0; i < nn * size_t(NS > 0 ? NS : 1); ++i) cidx[i] = -1;
  for (int s = 0; s < NS; ++s) std::fill(ext[s], ext[s] + 3 * sc->sensors[s].nv, T(0));

  // ---- compute_new_F + svd + p2g ----
#pragma omp parallel for num_threads(nt) schedule(static) reduction(| : err) if (at)
  for (int p = 0; p < sc->n_particles; ++p) {
    Particle<T> q = load_particle(x, v, C, F, p);
    P2GFwd<T> o;
    if (!particle_base(sc, K, q.x, o.base, o.fx)) {
      err |= 1;
      for (int i = 0; i < 9; ++i) F1[9 * p + i] = F[9 * p + i];
      continue;
    }
    p2g_particle(sc, K, q, p, o);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const int off[3] = {i, j, k};
          T dpos[3];
          for (int d = 0; d < 3; ++d) dpos[d] = (T(off[d]) - o.fx[d]) * K.dx;
          T W = (o.w[i][0] * o.w[j][1]) * o.w[k][2];
          size_t g = gidx(n, o.base[0] + i, o.base[1] + j, o.base[2] + k);
          for (int r = 0; r < 3; ++r) {
            T ad = o.affine.a[r][0] * dpos[0];
            ad = ad + o.affine.a[r][1] * dpos[1];
            ad = ad + o.affine.a[r][2] * dpos[2];
            aadd(grid_v_in[3 * g + r], W * (K.p_mass * q.v[r] + ad), at);
          }
          aadd(grid_m[g], W * K.p_mass, at);
        }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) F1[9 * p + 3 * i + j] = o.Fp.a[i][j];
  }

  // ---- FEM update (fem_sensor.py:409-440) ----
  for (int s = 0; s < NS; ++s) {
    const orc_sensor& S = sc->sensors[s];
    const T dt = T(sc->dt), mass = T(S.mass), mu = T(S.mu), lam = T(S.lam);
    const T alpha = T(1) + T(0.75) * mu / lam;
    T* P = pos[s];
    T* Vl = vel[s];
#pragma omp parallel for num_threads(nt) schedule(static) if (at)
    for (int t = 0; t < S.nt; ++t) {
      const int* tv = S.tets + 4 * t;
      M3<T> D, B;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          D.a[r][c] = P[3 * tv[c] + r] - P[3 * tv[3] + r];
          B.a[r][c] = T(S.B[9 * t + 3 * r + c]);
        }
      T Vi = std::fabs(mdet(D)) / T(6);
      M3<T> Fe = mmul(D, B);
      M3<T> Pk;
      if (S.model == 1) {
        // linear corotated: P = 2 mu (F - R) + lam tr(R^T F - I) R with F = R S (R = U V^T of the SVD,
        // tr(R^T F) = sum sigma), weighted by the rest volume 1 / (6 |det B|)
        M3<T> U, Vs;
        T sg[3];
        svd3(Fe, U, sg, Vs, sc->svd_sweeps);
        const M3<T> R = mmul(U, mT(Vs));
        const T c = ((sg[0] + sg[1]) + sg[2]) - T(3);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Pk.a[i][j] = T(2) * mu * (Fe.a[i][j] - R.a[i][j]) + lam * c * R.a[i][j];
        Vi = T(1) / (T(6) * std::fabs(mdet(B)));
      } else {
        T J = mdet(Fe);
        T IC = T(0);
        for (int i = 0; i < 3; ++i) {
          T cc = Fe.a[0][i] * Fe.a[0][i];
          cc = cc + Fe.a[1][i] * Fe.a[1][i];
          cc = cc + Fe.a[2][i] * Fe.a[2][i];
          IC = IC + cc;
        }
        M3<T> cof = mcof(Fe);  // columns: F1xF2, F2xF0, F0xF1
        T k1 = mu * (T(1) - T(1) / (IC + T(1)));
        T k2 = lam * (J - alpha);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Pk.a[i][j] = k1 * Fe.a[i][j] + k2 * cof.a[i][j];
      }
      M3<T> H = mmul(Pk, mT(B));
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H.a[i][j] = -Vi * H.a[i][j];
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r) {
          T fo = H.a[r][k];
          aadd(Vl[3 * tv[k] + r], dt * fo / mass, at);
          aadd(Vl[3 * tv[3] + r], T(-1) * dt * fo / mass, at);
        }
    }
  }

  // ---- check_grid_occupy + check_collision + collision + grid_op ----
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1) if (at)
  for (int i = 0; i < n[0]; ++i)
    for (int j = 0; j < n[1]; ++j)
      for (int k = 0; k < n[2]; ++k) {
        size_t g = gidx(n, i, j, k);
        T m = grid_m[g];
        if (!(m > K.eps)) continue;
        T p[3] = {(T(i) + T(0.5)) * K.dx, (T(j) + T(0.5)) * K.dx, (T(k) + T(0.5)) * K.dx};
        T cur_v[3];
        for (int c = 0; c < 3; ++c) cur_v[c] = grid_v_in[3 * g + c] / (m + K.eps);
        for (int s = 0; s < NS; ++s) {
          const orc_sensor& S = sc->sensors[s];
          int kk = find_closest(S, pos[s], p);
          cidx[g * NS + s] = kk;
          if (kk < 0) continue;
          SdfOut<T> so = find_sdf(S, pos[s], vel[s], kk, p, cur_v);
          if (!so.flag) continue;
          T e[3];
          contact_force(K, so.sdf, so.nrm, so.rel, e);
          for (int c = 0; c < 3; ++c) grid_f[3 * g + c] += e[c] * K.dt;
          const int* t = S.tris + 3 * kk;
          for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) aadd(ext[s][3 * t[a] + c], K.third * (T(-1) * e[c]), at);
        }
        T inv_m = T(1) / (m + K.eps);
        T vo[3];
        for (int c = 0; c < 3; ++c) {
          T a = T(0) + inv_m * grid_v_in[3 * g + c];
          a = a + inv_m * grid_f[3 * g + c];
          vo[c] = a + K.dt_g[c];
        }
        const int idx[3] = {i, j, k};
        for (int d = 0; d < 3; ++d) {
          if (idx[d] < sc->bound && vo[d] < T(0)) vo[d] = T(0);
          if (idx[d] > n[d] - sc->bound && vo[d] > T(0)) vo[d] = T(0);
        }
        if (sc->bc == 1 && j < sc->bound) vo[0] = vo[1] = vo[2] = T(0);
        for (int c = 0; c < 3; ++c) grid_v_out[3 * g + c] = vo[c];
      }

  // ---- PBD ropes ----
  for (int r = 0; r < sc->n_ropes; ++r) rope_fwd<T>(sc, sc->ropes[r], sc->rope_io[r], pos, vel, ext);

  // ---- g2p ----
#pragma omp parallel for num_threads(nt) schedule(static) if (at)
  for (int p = 0; p < sc->n_particles; ++p) {
    T xp[3];
    for (int d = 0; d < 3; ++d) xp[d] = x[3 * p + d];
    int base[3];
    T fx[3];
    if (!particle_base(sc, K, xp, base, fx)) {
      for (int d = 0; d < 3; ++d) {
        x1[3 * p + d] = x[3 * p + d];
        v1[3 * p + d] = v[3 * p + d];
      }
      for (int i = 0; i < 9; ++i) C1[9 * p + i] = C[9 * p + i];
      continue;
    }
    T w[3][3], dw[3][3];
    for (int d = 0; d < 3; ++d) {
      T wd[3], dwd[3];
      bspline(fx[d], wd, dwd);
      for (int i = 0; i < 3; ++i) {
        w[i][d] = wd[i];
        dw[i][d] = dwd[i];
      }
    }
    T nv[3] = {T(0), T(0), T(0)};
    M3<T> nC = mzero<T>();
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const int off[3] = {i, j, k};
          T dpos[3];
          for (int d = 0; d < 3; ++d) dpos[d] = T(off[d]) - fx[d];
          size_t g = gidx(n, base[0] + i, base[1] + j, base[2] + k);
          const T* gv = grid_v_out + 3 * g;
          T W = (w[i][0] * w[j][1]) * w[k][2];
          T kw = K.g2p_k * W;
          for (int r = 0; r < 3; ++r) {
            nv[r] += W * gv[r];
            for (int c = 0; c < 3; ++c) nC.a[r][c] += kw * (gv[r] * dpos[c]);
          }
        }
    for (int d = 0; d < 3; ++d) {
      v1[3 * p + d] = nv[d];
      x1[3 * p + d] = xp[d] + K.dt * nv[d];
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) C1[9 * p + 3 * i + j] = nC.a[i][j];
  }

  // ---- FEM update2 (fem_sensor.py:444-457, gripper_fem.py:404-418) ----
  for (int s = 0; s < NS; ++s) {
    const orc_sensor& S = sc->sensors[s];
    const T dt = T(sc->dt), mass = T(S.mass);
    for (int i = 0; i < S.nv; ++i) {
      T vo[3];
      for (int c = 0; c < 3; ++c) vo[c] = (T(0) + vel[s][3 * i + c]) + dt * ext[s][3 * i + c] / mass;
      if (S.layer[i] == 0)
        for (int c = 0; c < 3; ++c) vo[c] = cv[s][3 * i + c];
      for (int c = 0; c < 3; ++c) {
        T carry = S.carry ? (cv1[s][3 * i + c] - cv[s][3 * i + c]) : T(0);
        vel1[s][3 * i + c] = vo[c] + carry;
        pos1[s][3 * i + c] = pos[s][3 * i + c] + dt * vo[c];
        vpos1[s][3 * i + c] = vpos[s][3 * i + c] + dt * cv[s][3 * i + c];
      }
    }
  }
  return err;
}

// =============================================================================================
// Adjoint substep, order of Contact.update_grad (grasp_plastic.py:167-178): fem.update2.grad,
// g2p.grad, grid_op.grad, clamp_grid, collision.grad (argmin held constant), fem.update.grad,
// p2g.grad, svd_grad (mpm_elastic.py:145-173), compute_new_F.grad.  Recomputes the forward
// substep internally.  Adjoint inputs are those of frame f+1; outputs those of frame f; cvb, cvb1
// (control-velocity adjoints of frames f, f+1) and mat_b ([n_materials][2]: d/dmu, d/dlam) are
// accumulated.
// =============================================================================================
template <typename T>
inline T clampg(T a, T c) {
  return c > T(0) ? std::min(std::max(a, -c), c) : a;
}
// c (y^p - x^p) / (y - x) for x, y > 0 from fx = c x^p, fy = c y^p, gx = c x^(p-1): the quotient,
// or its series in t = (y - x) / x where the two are within 1%
template <typename T>
inline T cdd(T x, T y, T fx, T fy, T gx, T p) {
  const T h = y - x;
  if (std::fabs(h) > T(1e-2) * std::max(x, y)) return (fy - fx) / h;
  const T t = h / x, q = p - T(1);
  return p * gx * (T(1) + t * (T(0.5) * q + t * (q * (q - T(1)) / T(6) + t * (q * (q - T(1)) * (q - T(2)) / T(24)))));
}
template <typename T>
inline T gap_clamp(T a) {
  return a >= T(0) ? std::max(a, T(1e-8)) : std::min(a, T(-1e-8));
}

// adjoint of contact_force: returns sdf_b, accumulates n_b, r_b
template <typename T>
T contact_force_bwd(const Consts<T>& K, T sdf, const T n[3], const T r[3], const T eb[3], T nb[3], T rb[3]) {
  T nr = dot3(n, r);
  T vn = K.clamp_vn ? std::max(nr, T(0)) : nr;
  T kk = K.kn + K.kd * vn;
  T fn[3], vt[3];
  for (int c = 0; c < 3; ++c) {
    fn[c] = -kk * sdf * n[c];
    vt[c] = r[c] - nr * n[c];
  }
  T vtn = std::sqrt(dot3(vt, vt) + T(1e-11));
  T fnb[3] = {eb[0], eb[1], eb[2]};
  T vtb[3] = {T(0), T(0), T(0)};
  if (vtn > T(1e-4)) {
    T fnn = std::sqrt(dot3(fn, fn));
    T kv = K.kt * vtn, cap = K.mu_t * fnn;
    T g = std::min(kv, cap);
    T th[3] = {vt[0] / vtn, vt[1] / vtn, vt[2] / vtn};
    T gb = dot3(th, eb);
    T thb[3] = {g * eb[0], g * eb[1], g * eb[2]};
    T vtnb = T(0);
    if (kv <= cap)
      vtnb += K.kt * gb;
    else if (fnn > T(0))
      for (int c = 0; c < 3; ++c) fnb[c] += (K.mu_t * gb / fnn) * fn[c];
    for (int c = 0; c < 3; ++c) vtb[c] = thb[c] / vtn;
    vtnb += -dot3(thb, vt) / (vtn * vtn);
    for (int c = 0; c < 3; ++c) vtb[c] += (vtnb / vtn) * vt[c];
  }
  T nrb = -dot3(n, vtb);
  for (int c = 0; c < 3; ++c) {
    rb[c] += vtb[c];
    nb[c] -= nr * vtb[c];
  }
  T nfb = dot3(n, fnb);
  T kkb = -sdf * nfb;
  T sdfb = -kk * nfb;
  for (int c = 0; c < 3; ++c) nb[c] -= (kk * sdf) * fnb[c];
  if (!K.clamp_vn || nr > T(0)) nrb += K.kd * kkb;
  for (int c = 0; c < 3; ++c) {
    nb[c] += nrb * r[c];
    rb[c] += nrb * n[c];
  }
  return sdfb;
}

template <typename T>
M3<T> svd_grad(const M3<T>& U, const T s[3], const M3<T>& V, const M3<T>& Ub0, const T sb[3], const M3<T>& Vb0,
               const M3<T>& Rb, int mode) {
  M3<T> Ub = Ub0, Vb = Vb0;
  if (mode == 1) {
    M3<T> a = mmul(Rb, V), b = mmul(mT(Rb), U);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Ub.a[i][j] += a.a[i][j];
        Vb.a[i][j] += b.a[i][j];
      }
  }
  M3<T> M = mmul(mmul(mT(U), Rb), V);
  M3<T> UtUb = mmul(mT(U), Ub), UbtU = mmul(mT(Ub), U), VtVb = mmul(mT(V), Vb), VbtV = mmul(mT(Vb), V);
  M3<T> inner;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T val;
      if (i != j) {
        T ff = T(1) / gap_clamp(s[j] * s[j] - s[i] * s[i]);
        val = ff * (UtUb.a[i][j] - UbtU.a[i][j]) * s[j] + s[i] * ff * (VtVb.a[i][j] - VbtV.a[i][j]);
        if (mode != 1) val += (M.a[i][j] - M.a[j][i]) / gap_clamp(s[i] + s[j]);
      } else {
        val = sb[i];
      }
      inner.a[i][j] = val;
    }
  return mmul(mmul(U, inner), mT(V));
}

// adjoint of the sensor-triangle geometry of find_sdf (normal and sdf) for a contact at point p:
// accumulates the triangle vertices' position adjoints
template <typename T>
void tri_geom_bwd(const orc_sensor& S, const T* pos, int kk, const T p[3], const SdfOut<T>& so, T sdfb, T nb[3],
                  T* posb) {
  const int* t = S.tris + 3 * kk;
  const T* p1 = pos + 3 * t[0];
  const T* p2 = pos + 3 * t[1];
  const T* p3 = pos + 3 * t[2];
  T p1b[3], e1[3], e2[3], nrm[3];
  for (int c = 0; c < 3; ++c) {
    p1b[c] = -sdfb * so.nrm[c];
    nb[c] += sdfb * (p[c] - p1[c]);
    e1[c] = p2[c] - p1[c];
    e2[c] = p3[c] - p1[c];
  }
  cross(e1, e2, nrm);
  T L = std::sqrt(dot3(nrm, nrm));
  T od[3] = {T(S.out_dir[0]), T(S.out_dir[1]), T(S.out_dir[2])};
  T inv = T(1) / (L + T(1e-10));
  T nn_[3] = {inv * nrm[0], inv * nrm[1], inv * nrm[2]};
  T sg = dot3(nn_, od) < T(0) ? T(-1) : T(1);
  T nrmb[3] = {T(0), T(0), T(0)};
  if (L > T(0)) {
    T D = L + T(1e-10);
    T q = dot3(nb, nrm) / (D * D * L);
    for (int c = 0; c < 3; ++c) nrmb[c] = sg * (nb[c] / D - q * nrm[c]);
  }
  T e1b[3], e2b[3];
  cross(e2, nrmb, e1b);
  cross(nrmb, e1, e2b);
  for (int c = 0; c < 3; ++c) {
    posb[3 * t[0] + c] += p1b[c] - (e1b[c] + e2b[c]);
    posb[3 * t[1] + c] += e1b[c];
    posb[3 * t[2] + c] += e2b[c];
  }
}

// adjoint of one Jacobi pass: tp_out = tp_in + dp(tp_in); tpb holds d/d tp_out on entry and
// d/d tp_in on return
template <typename T>
void rope_pass_bwd(const std::vector<T>& tp_in, std::vector<T>& tpb, int n, int stride, T len, T alpha, T relax,
                   T w) {
  std::vector<T> add(3 * n, T(0));
  const T k = -relax / (w + w + alpha);
  for (int e = 0; e + stride < n; ++e) {
    const T* x1 = &tp_in[3 * e];
    const T* x2 = &tp_in[3 * (e + stride)];
    T d[3] = {x1[0] - x2[0], x1[1] - x2[1], x1[2] - x2[2]};
    T L = std::sqrt(dot3(d, d) + T(1e-10));
    // dp = k (L - len) / L d, applied +w at e and -w at e + stride
    T dpb[3];
    for (int c = 0; c < 3; ++c) dpb[c] = w * (tpb[3 * e + c] - tpb[3 * (e + stride) + c]);
    T a = k * (L - len) / L;
    T dd = dot3(d, dpb);
    T bcoef = k * len / (L * L * L) * dd;
    for (int c = 0; c < 3; ++c) {
      T db = a * dpb[c] + bcoef * d[c];
      add[3 * e + c] += db;
      add[3 * (e + stride) + c] -= db;
    }
  }
  for (int i = 0; i < 3 * n; ++i) tpb[i] += add[i];
}

// adjoint of rope_fwd (order of cable_straightening.py:177-186: rope.update.grad, clamp_grid, then
// collision.grad).  The forward has been recomputed (io.ext, io.cidx hold its values); exb are the
// sensors' external-force adjoints; vmb / posb the sensors' velmid / position adjoints (accumulated).
template <typename T>
void rope_bwd(const orc_scene* sc, const orc_rope& R, orc_rope_io& io, T* const* pos, T* const* vel_mid,
              const std::vector<std::vector<T>>& exb, std::vector<std::vector<T>>& vmb, T* const* posb, T clip) {
  const int n = R.n, NS = sc->n_sensors;
  const T dt = T(sc->dt);
  const Consts<T> K = rope_consts<T>(sc, R);
  const T* rp = static_cast<const T*>(io.pos);
  const T* rv = static_cast<const T*>(io.vel);
  const T* re = static_cast<const T*>(io.ext);
  const T* pb1 = static_cast<const T*>(io.posb1);
  const T* vb1 = static_cast<const T*>(io.velb1);
  const T* tb1 = static_cast<const T*>(io.travb1);
  T* rpb = static_cast<T*>(io.posb);
  T* rvb = static_cast<T*>(io.velb);
  T* rtb = static_cast<T*>(io.travb);
  const T w = T(1) / T(R.mass);
  std::vector<T> tp0;
  std::vector<unsigned char> fl;
  rope_integrate(R, dt, rp, rv, re, tp0, fl);
  // the input positions of every pass, recomputed: ins[2 it] stretch, ins[2 it + 1] bending
  const int iters = std::max(R.iters, 1);
  std::vector<std::vector<T>> ins(2 * iters);
  {
    std::vector<T> tp = tp0;
    for (int it = 0; it < iters; ++it) {
      ins[2 * it] = tp;
      rope_pass(tp, n, 1, T(R.rest), T(R.alpha_s), T(R.relax_s), w);
      ins[2 * it + 1] = tp;
      rope_pass(tp, n, 2, T(R.bend), T(R.alpha_b), T(R.relax_b), w);
    }
  }
  // vel1 = (pos1 - pos) / dt; pos1[0] = pin, pos1[i] = tp2[i]
  std::vector<T> tpb(3 * n, T(0));
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      const int q = 3 * i + c;
      T p1b = pb1[q] + vb1[q] / dt;
      rpb[q] = -vb1[q] / dt;
      tpb[q] = i == 0 ? T(0) : p1b;
    }
  for (int it = iters - 1; it >= 0; --it) {
    rope_pass_bwd(ins[2 * it + 1], tpb, n, 2, T(R.bend), T(R.alpha_b), T(R.relax_b), w);
    rope_pass_bwd(ins[2 * it], tpb, n, 1, T(R.rest), T(R.alpha_s), T(R.relax_s), w);
  }
  std::vector<T> reb(3 * n);
  for (int i = 0; i < n; ++i) {
    T nvb[3];
    for (int c = 0; c < 3; ++c) {
      rpb[3 * i + c] += tpb[3 * i + c];
      nvb[c] = tpb[3 * i + c] * dt;
    }
    if (fl[i]) {
      nvb[0] *= T(R.friction);
      nvb[1] = T(0);
      nvb[2] *= T(R.friction);
    }
    for (int c = 0; c < 3; ++c) {
      rvb[3 * i + c] = nvb[c];
      reb[3 * i + c] = nvb[c] / T(R.mass);
    }
  }
  // clamp_grid on the rope's frame-f grads (cable_straightening.py:196-199)
  for (int q = 0; q < 3 * n; ++q) {
    rpb[q] = clampg(rpb[q], clip);
    rvb[q] = clampg(rvb[q], clip);
  }
  // collision.grad (argmin held constant)
  for (int p = 0; p < n; ++p) {
    bool any = false;
    for (int s = 0; s < NS; ++s) {
      const orc_sensor& S = sc->sensors[s];
      const int kk = io.cidx[p * NS + s];
      if (kk < 0) continue;
      SdfOut<T> so = find_sdf(S, pos[s], vel_mid[s], kk, rp + 3 * p, rv + 3 * p, T(R.rad));
      if (!so.flag) continue;
      any = true;
      const int* t = S.tris + 3 * kk;
      T eb[3];
      for (int c = 0; c < 3; ++c)
        eb[c] = dt * reb[3 * p + c] - K.third * ((exb[s][3 * t[0] + c] + exb[s][3 * t[1] + c]) + exb[s][3 * t[2] + c]);
      T nb[3] = {T(0), T(0), T(0)}, rb[3] = {T(0), T(0), T(0)};
      T sdfb = contact_force_bwd(K, so.sdf, so.nrm, so.rel, eb, nb, rb);
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) vmb[s][3 * t[a] + c] += K.third * rb[c];
      for (int c = 0; c < 3; ++c) {
        rvb[3 * p + c] -= rb[c];
        rpb[3 * p + c] += sdfb * so.nrm[c];
      }
      tri_geom_bwd(S, pos[s], kk, rp + 3 * p, so, sdfb, nb, posb[s]);
    }
    rtb[p] = any ? T(0) : tb1[p];
  }
}

template <typename T>
static int substep_bwd_impl(const orc_scene* sc, const T* x, const T* v, const T* C, const T* F,
                            const T* const* pos, const T* const* vel, const T* const* vpos, const T* const* cv,
                            const T* const* cv1, const T* xb1, const T* vb1, const T* Cb1, const T* Fb1,
                            const T* const* posb1, const T* const* velb1, const T* const* vpb1, T* xb, T* vb, T* Cb,
                            T* Fb, T* const* posb, T* const* velb, T* const* vpb, T* const* cvb, T* const* cvb1,
                            T* mat_b, int svd_grad_mode) {
  const Consts<T> K = make_consts<T>(sc);
  const int* n = sc->n;
  const size_t nn = size_t(n[0]) * n[1] * n[2];
  const int NS = sc->n_sensors;
  const int Np = sc->n_particles;
  const int nt = sc->n_threads > 1 ? sc->n_threads : 1;
  const bool at = nt > 1;
  const T clip = T(sc->grad_clip);
  // ---- forward recompute ----
  std::vector<T> x1(3 * Np), v1(3 * Np), C1(9 * Np), F1(9 * Np);
  std::vector<std::vector<T>> pos_c(NS), vel_c(NS), p1(NS), vl1(NS), vp1(NS), ext(NS);
  std::vector<T*> pos_p(NS), vel_p(NS), p1_p(NS), vl1_p(NS), vp1_p(NS), ext_p(NS);
  for (int s = 0; s < NS; ++s) {
    const int nv = sc->sensors[s].nv;
    pos_c[s].assign(pos[s], pos[s] + 3 * nv);
    vel_c[s].assign(vel[s], vel[s] + 3 * nv);
    p1[s].resize(3 * nv);
    vl1[s].resize(3 * nv);
    vp1[s].resize(3 * nv);
    ext[s].resize(3 * nv);
    pos_p[s] = pos_c[s].data();
    vel_p[s] = vel_c[s].data();
    p1_p[s] = p1[s].data();
    vl1_p[s] = vl1[s].data();
    vp1_p[s] = vp1[s].data();
    ext_p[s] = ext[s].data();
  }
  std::vector<T> gm(nn), gvi(3 * nn), gvo(3 * nn), gf(3 * nn);
  std::vector<int> cid(nn * size_t(NS > 0 ? NS : 1));
  substep_impl<T>(sc, x, v, C, F, x1.data(), v1.data(), C1.data(), F1.data(), pos_p.data(), vel_p.data(), vpos, cv,
                  cv1, p1_p.data(), vl1_p.data(), vp1_p.data(), ext_p.data(), gm.data(), gvi.data(), gvo.data(),
                  gf.data(), cid.data());
  // vel_c now holds the post-elastic-force velocities (vel_mid)

  // ---- fem.update2.grad + clamp_grid on the sensor grads ----
  std::vector<std::vector<T>> vmb(NS), exb(NS);
  for (int s = 0; s < NS; ++s) {
    const orc_sensor& S = sc->sensors[s];
    const T dt = T(sc->dt), mass = T(S.mass);
    vmb[s].assign(3 * S.nv, T(0));
    exb[s].assign(3 * S.nv, T(0));
    for (int i = 0; i < S.nv; ++i)
      for (int c = 0; c < 3; ++c) {
        const int q = 3 * i + c;
        vpb[s][q] = vpb1[s][q];
        cvb[s][q] += dt * vpb1[s][q];
        T vob = velb1[s][q] + dt * posb1[s][q];
        if (S.carry) {
          cvb1[s][q] += velb1[s][q];
          cvb[s][q] -= velb1[s][q];
        }
        if (S.layer[i] == 0) {
          cvb[s][q] += vob;
        } else {
          vmb[s][q] = vob;
          exb[s][q] = dt * vob / mass;
        }
        posb[s][q] = clampg(posb1[s][q], clip);
        vmb[s][q] = clampg(vmb[s][q], clip);
      }
  }

  // ---- PBD ropes: update.grad, clamp_grid, collision.grad ----
  for (int r = 0; r < sc->n_ropes; ++r)
    rope_bwd<T>(sc, sc->ropes[r], sc->rope_io[r], pos_p.data(), vel_p.data(), exb, vmb, posb, clip);

  // ---- g2p.grad ----
  std::vector<T> gvb(3 * nn, T(0));
#pragma omp parallel for num_threads(nt) schedule(static) if (at)
  for (int p = 0; p < Np; ++p) {
    T xp[3];
    for (int d = 0; d < 3; ++d) xp[d] = x[3 * p + d];
    int base[3];
    T fx[3];
    if (!particle_base(sc, K, xp, base, fx)) {
      for (int d = 0; d < 3; ++d) {
        xb[3 * p + d] = xb1[3 * p + d];
        vb[3 * p + d] = vb1[3 * p + d];
      }
      for (int i = 0; i < 9; ++i) {
        Cb[9 * p + i] = Cb1[9 * p + i];
        Fb[9 * p + i] = Fb1[9 * p + i];
      }
      continue;
    }
    T w[3][3], dw[3][3];
    for (int d = 0; d < 3; ++d) {
      T wd[3], dwd[3];
      bspline(fx[d], wd, dwd);
      for (int i = 0; i < 3; ++i) {
        w[i][d] = wd[i];
        dw[i][d] = dwd[i];
      }
    }
    T vnb[3], fxb[3] = {T(0), T(0), T(0)};
    for (int d = 0; d < 3; ++d) vnb[d] = vb1[3 * p + d] + K.dt * xb1[3 * p + d];
    const T* Cbp = Cb1 + 9 * p;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const int off[3] = {i, j, k};
          T d[3];
          for (int c = 0; c < 3; ++c) d[c] = T(off[c]) - fx[c];
          size_t g = gidx(n, base[0] + i, base[1] + j, base[2] + k);
          const T* gv = gvo.data() + 3 * g;
          T W = (w[i][0] * w[j][1]) * w[k][2];
          T kw = K.g2p_k * W;
          T Cd[3], Ctg[3];
          for (int r = 0; r < 3; ++r) {
            Cd[r] = Cbp[3 * r] * d[0] + Cbp[3 * r + 1] * d[1] + Cbp[3 * r + 2] * d[2];
            Ctg[r] = Cbp[r] * gv[0] + Cbp[3 + r] * gv[1] + Cbp[6 + r] * gv[2];
          }
          for (int r = 0; r < 3; ++r) aadd(gvb[3 * g + r], W * vnb[r] + kw * Cd[r], at);
          T Wb = dot3(gv, vnb) + K.g2p_k * dot3(gv, Cd);
          fxb[0] += Wb * (dw[i][0] * w[j][1] * w[k][2]) - kw * Ctg[0];
          fxb[1] += Wb * (w[i][0] * dw[j][1] * w[k][2]) - kw * Ctg[1];
          fxb[2] += Wb * (w[i][0] * w[j][1] * dw[k][2]) - kw * Ctg[2];
        }
    for (int d = 0; d < 3; ++d) xb[3 * p + d] = xb1[3 * p + d] + K.inv_dx * fxb[d];
  }

  // ---- grid_op.grad + clamp_grid + collision.grad ----
  std::vector<T> accb(4 * nn, T(0));
  for (int i = 0; i < n[0]; ++i)
    for (int j = 0; j < n[1]; ++j)
      for (int k = 0; k < n[2]; ++k) {
        size_t g = gidx(n, i, j, k);
        T m = gm[g];
        if (!(m > K.eps)) continue;
        const T me = m + K.eps, inv_m = T(1) / me;
        const T* mv = gvi.data() + 3 * g;
        T cur_v[3] = {mv[0] / me, mv[1] / me, mv[2] / me};
        T u[3];
        for (int c = 0; c < 3; ++c) u[c] = (T(0) + inv_m * mv[c]) + inv_m * gf[3 * g + c] + K.dt_g[c];
        const int idx[3] = {i, j, k};
        bool mask[3];
        for (int d = 0; d < 3; ++d)
          mask[d] = (idx[d] < sc->bound && u[d] < T(0)) || (idx[d] > n[d] - sc->bound && u[d] > T(0));
        if (sc->bc == 1 && j < sc->bound) mask[0] = mask[1] = mask[2] = true;
        T ub[3], mvb[3], gfb[3];
        for (int c = 0; c < 3; ++c) {
          ub[c] = mask[c] ? T(0) : gvb[3 * g + c];
          mvb[c] = inv_m * ub[c];
          gfb[c] = inv_m * ub[c];
        }
        T invb = ub[0] * (mv[0] + gf[3 * g + 0]) + ub[1] * (mv[1] + gf[3 * g + 1]) + ub[2] * (mv[2] + gf[3 * g + 2]);
        T mb = clampg(-inv_m * inv_m * invb, clip);
        T p[3] = {(T(i) + T(0.5)) * K.dx, (T(j) + T(0.5)) * K.dx, (T(k) + T(0.5)) * K.dx};
        T curvb[3] = {T(0), T(0), T(0)};
        for (int s = 0; s < NS; ++s) {
          const orc_sensor& S = sc->sensors[s];
          const int kk = cid[g * NS + s];
          if (kk < 0) continue;
          SdfOut<T> so = find_sdf(S, pos[s], vel_c[s].data(), kk, p, cur_v);
          if (!so.flag) continue;
          const int* t = S.tris + 3 * kk;
          T eb[3];
          for (int c = 0; c < 3; ++c)
            eb[c] = K.dt * gfb[c] - K.third * ((exb[s][3 * t[0] + c] + exb[s][3 * t[1] + c]) + exb[s][3 * t[2] + c]);
          T nb[3] = {T(0), T(0), T(0)}, rb[3] = {T(0), T(0), T(0)};
          T sdfb = contact_force_bwd(K, so.sdf, so.nrm, so.rel, eb, nb, rb);
          for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) vmb[s][3 * t[a] + c] += K.third * rb[c];
          for (int c = 0; c < 3; ++c) curvb[c] -= rb[c];
          const T* p1 = pos[s] + 3 * t[0];
          const T* p2 = pos[s] + 3 * t[1];
          const T* p3 = pos[s] + 3 * t[2];
          T p1b[3], e1[3], e2[3], nrm[3];
          for (int c = 0; c < 3; ++c) {
            p1b[c] = -sdfb * so.nrm[c];
            nb[c] += sdfb * (p[c] - p1[c]);
            e1[c] = p2[c] - p1[c];
            e2[c] = p3[c] - p1[c];
          }
          cross(e1, e2, nrm);
          T L = std::sqrt(dot3(nrm, nrm));
          T od[3] = {T(S.out_dir[0]), T(S.out_dir[1]), T(S.out_dir[2])};
          T inv = T(1) / (L + T(1e-10));
          T nn_[3] = {inv * nrm[0], inv * nrm[1], inv * nrm[2]};
          T sg = dot3(nn_, od) < T(0) ? T(-1) : T(1);
          T nrmb[3] = {T(0), T(0), T(0)};
          if (L > T(0)) {
            T D = L + T(1e-10);
            T q = dot3(nb, nrm) / (D * D * L);
            for (int c = 0; c < 3; ++c) nrmb[c] = sg * (nb[c] / D - q * nrm[c]);
          }
          T e1b[3], e2b[3];
          cross(e2, nrmb, e1b);
          cross(nrmb, e1, e2b);
          for (int c = 0; c < 3; ++c) {
            posb[s][3 * t[0] + c] += p1b[c] - (e1b[c] + e2b[c]);
            posb[s][3 * t[1] + c] += e1b[c];
            posb[s][3 * t[2] + c] += e2b[c];
          }
        }
        for (int c = 0; c < 3; ++c) {
          accb[4 * g + c] = mvb[c] + inv_m * curvb[c];
        }
        accb[4 * g + 3] = mb - dot3(curvb, mv) * inv_m * inv_m;
      }

  // ---- fem.update.grad ----
  for (int s = 0; s < NS; ++s) {
    const orc_sensor& S = sc->sensors[s];
    const T dt = T(sc->dt), mass = T(S.mass), mu = T(S.mu), lam = T(S.lam);
    const T alpha = T(1) + T(0.75) * mu / lam;
    const T* P = pos[s];
    for (int t = 0; t < S.nt; ++t) {
      const int* tv = S.tets + 4 * t;
      M3<T> D, B;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          D.a[r][c] = P[3 * tv[c] + r] - P[3 * tv[3] + r];
          B.a[r][c] = T(S.B[9 * t + 3 * r + c]);
        }
      T detD = mdet(D);
      T Vi = std::fabs(detD) / T(6);
      M3<T> Fe = mmul(D, B);
      if (S.model == 1) {
        // linear corotated (see the forward): P = 2 mu (F - R) + lam c R, c = sum sigma - 3, rest volume
        M3<T> U, Vs;
        T sg[3];
        svd3(Fe, U, sg, Vs, sc->svd_sweeps);
        const M3<T> R = mmul(U, mT(Vs));
        const T c = ((sg[0] + sg[1]) + sg[2]) - T(3);
        const T V0 = T(1) / (T(6) * std::fabs(mdet(B)));
        const T sc_ = -V0 * dt / mass;
        M3<T> Hb;
        for (int k = 0; k < 3; ++k)
          for (int r = 0; r < 3; ++r) Hb.a[r][k] = sc_ * (vmb[s][3 * tv[k] + r] - vmb[s][3 * tv[3] + r]);
        const M3<T> Pb = mmul(Hb, B);  // H = P B^T
        M3<T> Fb_, Rb, zero = mzero<T>();
        T cb = T(0);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            Fb_.a[i][j] = T(2) * mu * Pb.a[i][j];
            Rb.a[i][j] = (lam * c - T(2) * mu) * Pb.a[i][j];
            cb += lam * Pb.a[i][j] * R.a[i][j];
          }
        const T sb[3] = {cb, cb, cb};  // d c / d sigma = 1
        const M3<T> g = svd_grad(U, sg, Vs, zero, sb, zero, Rb, svd_grad_mode);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Fb_.a[i][j] += g.a[i][j];
        M3<T> Db = mmul(Fb_, mT(B));
        for (int k = 0; k < 3; ++k)
          for (int r = 0; r < 3; ++r) {
            posb[s][3 * tv[k] + r] += Db.a[r][k];
            posb[s][3 * tv[3] + r] -= Db.a[r][k];
          }
        continue;
      }
      T J = mdet(Fe);
      T IC = T(0);
      for (int i = 0; i < 3; ++i)
        for (int r = 0; r < 3; ++r) IC += Fe.a[r][i] * Fe.a[r][i];
      M3<T> cof = mcof(Fe);
      T k1 = mu * (T(1) - T(1) / (IC + T(1)));
      T k2 = lam * (J - alpha);
      M3<T> Pk;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Pk.a[i][j] = k1 * Fe.a[i][j] + k2 * cof.a[i][j];
      M3<T> H = mmul(Pk, mT(B));
      const T sc_ = -Vi * dt / mass;
      M3<T> Hb;
      T scb = T(0);
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r) {
          T hb = vmb[s][3 * tv[k] + r] - vmb[s][3 * tv[3] + r];
          Hb.a[r][k] = sc_ * hb;
          scb += hb * H.a[r][k];
        }
      T Vib = -dt / mass * scb;
      M3<T> Pb = mmul(Hb, B);
      M3<T> Fb_;
      T k1b = T(0), k2b = T(0);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          Fb_.a[i][j] = k1 * Pb.a[i][j];
          k1b += Pb.a[i][j] * Fe.a[i][j];
          k2b += Pb.a[i][j] * cof.a[i][j];
        }
      T f[3][3], pb[3][3];
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r) {
          f[k][r] = Fe.a[r][k];
          pb[k][r] = Pb.a[r][k];
        }
      T g0[3], g1[3], g2[3], tmp[3];
      cross(pb[1], f[2], g0);
      cross(f[1], pb[2], tmp);
      for (int c = 0; c < 3; ++c) g0[c] += tmp[c];
      cross(f[2], pb[0], g1);
      cross(pb[2], f[0], tmp);
      for (int c = 0; c < 3; ++c) g1[c] += tmp[c];
      cross(pb[0], f[1], g2);
      cross(f[0], pb[1], tmp);
      for (int c = 0; c < 3; ++c) g2[c] += tmp[c];
      for (int r = 0; r < 3; ++r) {
        Fb_.a[r][0] += k2 * g0[r];
        Fb_.a[r][1] += k2 * g1[r];
        Fb_.a[r][2] += k2 * g2[r];
      }
      T ICb = k1b * mu / ((IC + T(1)) * (IC + T(1)));
      T Jb = lam * k2b;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Fb_.a[i][j] += T(2) * ICb * Fe.a[i][j] + Jb * cof.a[i][j];
      M3<T> Db = mmul(Fb_, mT(B));
      T sgn = detD < T(0) ? T(-1) : (detD > T(0) ? T(1) : T(0));
      M3<T> cD = mcof(D);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Db.a[i][j] += Vib * sgn / T(6) * cD.a[i][j];
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r) {
          posb[s][3 * tv[k] + r] += Db.a[r][k];
          posb[s][3 * tv[3] + r] -= Db.a[r][k];
        }
    }
    for (int q = 0; q < 3 * S.nv; ++q) velb[s][q] = vmb[s][q];
  }

  // ---- p2g.grad + svd_grad + compute_new_F.grad ----
#pragma omp parallel for num_threads(nt) schedule(static) if (at)
  for (int p = 0; p < Np; ++p) {
    Particle<T> q = load_particle(x, v, C, F, p);
    P2GFwd<T> o;
    if (!particle_base(sc, K, q.x, o.base, o.fx)) continue;  // passed through above
    p2g_particle(sc, K, q, p, o);
    const T pm = K.p_mass, dx = K.dx;
    T vbp[3] = {T(0), T(0), T(0)}, fxb[3] = {T(0), T(0), T(0)};
    M3<T> Ab = mzero<T>();
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const int off[3] = {i, j, k};
          size_t g = gidx(n, o.base[0] + i, o.base[1] + j, o.base[2] + k);
          const T* gb = accb.data() + 4 * g;
          T W = (o.w[i][0] * o.w[j][1]) * o.w[k][2];
          T dp[3];
          for (int c = 0; c < 3; ++c) dp[c] = (T(off[c]) - o.fx[c]) * dx;
          T Adp[3], Atm[3];
          for (int r = 0; r < 3; ++r) {
            Adp[r] = o.affine.a[r][0] * dp[0] + o.affine.a[r][1] * dp[1] + o.affine.a[r][2] * dp[2];
            Atm[r] = o.affine.a[0][r] * gb[0] + o.affine.a[1][r] * gb[1] + o.affine.a[2][r] * gb[2];
          }
          T Wb = pm * gb[3];
          for (int r = 0; r < 3; ++r) {
            vbp[r] += W * pm * gb[r];
            for (int c = 0; c < 3; ++c) Ab.a[r][c] += W * gb[r] * dp[c];
            Wb += gb[r] * (pm * q.v[r] + Adp[r]);
          }
          fxb[0] += Wb * (o.dw[i][0] * o.w[j][1] * o.w[k][2]) - dx * W * Atm[0];
          fxb[1] += Wb * (o.w[i][0] * o.dw[j][1] * o.w[k][2]) - dx * W * Atm[1];
          fxb[2] += Wb * (o.w[i][0] * o.w[j][1] * o.dw[k][2]) - dx * W * Atm[2];
        }
    M3<T> Cbp, G, Fpb, Ub = mzero<T>(), Vb = mzero<T>(), Rb = mzero<T>();
    M3<T> Frm = mzero<T>();  // the return map's rotation-part adjoint when formed directly
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Cbp.a[i][j] = pm * Ab.a[i][j];
        G.a[i][j] = K.stress_k * Ab.a[i][j];
        Fpb.a[i][j] = Fb1[9 * p + 3 * i + j];
      }
    T sb[3] = {T(0), T(0), T(0)};
    T Jb, mub = T(0), lamb = T(0);
    T trG = G.a[0][0] + G.a[1][1] + G.a[2][2];
    if (o.model == MODEL_NEOHOOKEAN) {
      M3<T> GGt, FFt = mmul(o.Fp, mT(o.Fp));
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) GGt.a[i][j] = G.a[i][j] + G.a[j][i];
      M3<T> t1 = mmul(GGt, o.Fp);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          Fpb.a[i][j] += o.mu * t1.a[i][j];
          mub += G.a[i][j] * (FFt.a[i][j] - (i == j ? T(1) : T(0)));
        }
      Jb = o.lam * trG / o.J;
      lamb = std::log(o.J) * trG;
    } else {
      M3<T> D;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D.a[i][j] = o.Fp.a[i][j] - o.R.a[i][j];
      M3<T> GF = mmul(G, o.Fp), GtD = mmul(mT(G), D), DFt = mmul(D, mT(o.Fp));
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          Fpb.a[i][j] += T(2) * o.mu * (GF.a[i][j] + GtD.a[i][j]);
          Rb.a[i][j] = T(-2) * o.mu * GF.a[i][j];
          mub += T(2) * G.a[i][j] * DFt.a[i][j];
        }
      Jb = o.lam * (T(2) * o.J - T(1)) * trG;
      lamb = o.J * (o.J - T(1)) * trG;
    }
    M3<T> Fnb;
    if (o.model == MODEL_COROTATED) {
      sb[0] += Jb * o.sig[1] * o.sig[2];
      sb[1] += Jb * o.sig[0] * o.sig[2];
      sb[2] += Jb * o.sig[0] * o.sig[1];
      Fnb = Fpb;
    } else {
      M3<T> cf = mcof(o.Fp);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Fpb.a[i][j] += Jb * cf.a[i][j];
      if (o.model == MODEL_VON_MISES && o.yield) {
        T ep[3], eh[3];
        for (int d = 0; d < 3; ++d) ep[d] = std::log(std::max(o.sig[d], T(0.05)));
        T mean = ((ep[0] + ep[1]) + ep[2]) / T(3);
        for (int d = 0; d < 3; ++d) eh[d] = ep[d] - mean;
        T nrm = std::sqrt(((eh[0] * eh[0] + eh[1] * eh[1]) + eh[2] * eh[2]) + T(1e-8));
        T dg = nrm - o.ys / (T(2) * o.mu);
        T rr = dg / nrm;
        T ex[3];
        for (int d = 0; d < 3; ++d) ex[d] = std::exp(ep[d] - rr * eh[d]);
        M3<T> UtFV = mmul(mmul(mT(o.U), Fpb), o.V), Ue = o.U, Ve = o.V;
        if (svd_grad_mode != 1 && o.sig[0] > T(0.05) && o.sig[1] > T(0.05) && o.sig[2] > T(0.05)) {
          // stable form (not in the reference): with e_k = c s_k^a the rotation part of the SVD
          // adjoint of Fp = U diag(e) V^T is, off the diagonal,
          // M_ij c dd(a+1) / (s_i + s_j) + M_ji c s_i s_j dd(a-1) / (s_i + s_j), dd the divided
          // difference of x^p; equal to the generic formula below wherever that one is finite
          // the powers from e itself: c s^(a+1) = e s, c s^(a-1) = e / s, c s^(a-2) = e / s^2
          const T a = T(1) - rr;
          const T* sg = o.sig;
          M3<T> inner = mzero<T>();
          for (int i = 0; i < 3; ++i)
            for (int j = i + 1; j < 3; ++j) {
              const T sum = sg[i] + sg[j];
              const T A = cdd(sg[i], sg[j], ex[i] * sg[i], ex[j] * sg[j], ex[i], a + T(1)) / sum;
              const T B = (sg[i] * sg[j]) * cdd(sg[i], sg[j], ex[i] / sg[i], ex[j] / sg[j], ex[i] / (sg[i] * sg[i]), a - T(1)) / sum;
              inner.a[i][j] = UtFV.a[i][j] * A + UtFV.a[j][i] * B;
              inner.a[j][i] = UtFV.a[j][i] * A + UtFV.a[i][j] * B;
            }
          Frm = mmul(mmul(o.U, inner), mT(o.V));
        } else {
          for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d) {
              Ue.a[i][d] *= ex[d];
              Ve.a[i][d] *= ex[d];
            }
          M3<T> a1 = mmul(Fpb, Ve), a2 = mmul(mT(Fpb), Ue);
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
              Ub.a[i][j] += a1.a[i][j];
              Vb.a[i][j] += a2.a[i][j];
            }
        }
        T epb[3], ehb[3], rrb = T(0);
        for (int d = 0; d < 3; ++d) epb[d] = UtFV.a[d][d] * ex[d];
        for (int d = 0; d < 3; ++d) {
          ehb[d] = -rr * epb[d];
          rrb -= epb[d] * eh[d];
        }
        T nrmb = rrb * o.ys / (T(2) * o.mu * nrm * nrm);
        mub += rrb * o.ys / (T(2) * o.mu * o.mu * nrm);
        for (int d = 0; d < 3; ++d) ehb[d] += nrmb * eh[d] / nrm;
        T mb_ = ((ehb[0] + ehb[1]) + ehb[2]) / T(3);
        for (int d = 0; d < 3; ++d) {
          T e_ = epb[d] + ehb[d] - mb_;
          sb[d] += o.sig[d] > T(0.05) ? e_ / o.sig[d] : T(0);
        }
        Fnb = mzero<T>();
      } else {
        Fnb = Fpb;
      }
    }
    if (o.model != MODEL_NEOHOOKEAN) {
      M3<T> gsv = svd_grad(o.U, o.sig, o.V, Ub, sb, Vb, Rb, svd_grad_mode);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Fnb.a[i][j] += gsv.a[i][j] + Frm.a[i][j];
    }
    M3<T> Ad = meye<T>();
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Ad.a[i][j] += K.dt * q.C.a[i][j];
    M3<T> Fbo = mmul(mT(Ad), Fnb), CFt = mmul(Fnb, mT(q.F));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Fb[9 * p + 3 * i + j] = Fbo.a[i][j];
        Cb[9 * p + 3 * i + j] = Cbp.a[i][j] + K.dt * CFt.a[i][j];
      }
    for (int d = 0; d < 3; ++d) {
      vb[3 * p + d] = vbp[d];
      xb[3 * p + d] += K.inv_dx * fxb[d];
    }
    const int m = sc->p_mat ? sc->p_mat[p] : 0;
    aadd(mat_b[2 * m], mub, at);
    aadd(mat_b[2 * m + 1], lamb, at);
  }
  return 0;
}

extern "C" {

int orc_substep_f32(const orc_scene* sc, const float* x, const float* v, const float* C, const float* F, float* x1,
                    float* v1, float* C1, float* F1, float* const* pos, float* const* vel, const float* const* vpos,
                    const float* const* cv, const float* const* cv1, float* const* pos1, float* const* vel1,
                    float* const* vpos1, float* const* ext, float* grid_m, float* grid_v_in, float* grid_v_out,
                    float* grid_f, int* cidx) {
  return substep_impl<float>(sc, x, v, C, F, x1, v1, C1, F1, pos, vel, vpos, cv, cv1, pos1, vel1, vpos1, ext, grid_m,
                             grid_v_in, grid_v_out, grid_f, cidx);
}

int orc_substep_f64(const orc_scene* sc, const double* x, const double* v, const double* C, const double* F,
                    double* x1, double* v1, double* C1, double* F1, double* const* pos, double* const* vel,
                    const double* const* vpos, const double* const* cv, const double* const* cv1,
                    double* const* pos1, double* const* vel1, double* const* vpos1, double* const* ext,
                    double* grid_m, double* grid_v_in, double* grid_v_out, double* grid_f, int* cidx) {
  return substep_impl<double>(sc, x, v, C, F, x1, v1, C1, F1, pos, vel, vpos, cv, cv1, pos1, vel1, vpos1, ext,
                              grid_m, grid_v_in, grid_v_out, grid_f, cidx);
}

// Standalone 3x3 SVD (for SVD-convention and accuracy tests): A, U, V [n][9], s [n][3].
void orc_svd3_f32(int n, const float* A, float* U, float* s, float* V, int sweeps) {
  for (int i = 0; i < n; ++i) {
    M3<float> a, u, v;
    std::memcpy(a.a, A + 9 * i, sizeof(a.a));
    svd3(a, u, s + 3 * i, v, sweeps);
    std::memcpy(U + 9 * i, u.a, sizeof(u.a));
    std::memcpy(V + 9 * i, v.a, sizeof(v.a));
  }
}
void orc_svd3_f64(int n, const double* A, double* U, double* s, double* V, int sweeps) {
  for (int i = 0; i < n; ++i) {
    M3<double> a, u, v;
    std::memcpy(a.a, A + 9 * i, sizeof(a.a));
    svd3(a, u, s + 3 * i, v, sweeps);
    std::memcpy(U + 9 * i, u.a, sizeof(u.a));
    std::memcpy(V + 9 * i, v.a, sizeof(v.a));
  }
}

// Standalone SVD adjoint (svd_grad, mpm_elastic.py:145-173, for finite-difference tests) in float64:
// U, V, Ub, Vb, Rb, Fb [n][9], s, sb [n][3]; Rb is the adjoint of R = U V^T (mode 1 folds it into Ub
// and Vb as the reference does, any other mode uses the divided form).
void orc_svd_grad_f64(int n, const double* U, const double* s, const double* V, const double* Ub,
                      const double* sb, const double* Vb, const double* Rb, int mode, double* Fb) {
  for (int i = 0; i < n; ++i) {
    M3<double> u, v, ub, vb, rb;
    std::memcpy(u.a, U + 9 * i, sizeof(u.a));
    std::memcpy(v.a, V + 9 * i, sizeof(v.a));
    std::memcpy(ub.a, Ub + 9 * i, sizeof(ub.a));
    std::memcpy(vb.a, Vb + 9 * i, sizeof(vb.a));
    std::memcpy(rb.a, Rb + 9 * i, sizeof(rb.a));
    M3<double> g = svd_grad(u, s + 3 * i, v, ub, sb + 3 * i, vb, rb, mode);
    std::memcpy(Fb + 9 * i, g.a, sizeof(g.a));
  }
}

// Standalone argmin (find_closest) over one sensor for a list of query points [nq][3].
void orc_find_closest_f32(const orc_sensor* s, const float* pos, int nq, const float* q, int* out) {
  for (int i = 0; i < nq; ++i) out[i] = find_closest(*s, pos, q + 3 * i);
}

int orc_substep_bwd_f32(const orc_scene* sc, const float* x, const float* v, const float* C, const float* F,
                        const float* const* pos, const float* const* vel, const float* const* vpos,
                        const float* const* cv, const float* const* cv1, const float* xb1, const float* vb1,
                        const float* Cb1, const float* Fb1, const float* const* posb1, const float* const* velb1,
                        const float* const* vpb1, float* xb, float* vb, float* Cb, float* Fb, float* const* posb,
                        float* const* velb, float* const* vpb, float* const* cvb, float* const* cvb1, float* mat_b,
                        int svd_grad_mode) {
  return substep_bwd_impl<float>(sc, x, v, C, F, pos, vel, vpos, cv, cv1, xb1, vb1, Cb1, Fb1, posb1, velb1, vpb1, xb,
                                 vb, Cb, Fb, posb, velb, vpb, cvb, cvb1, mat_b, svd_grad_mode);
}
int orc_substep_bwd_f64(const orc_scene* sc, const double* x, const double* v, const double* C, const double* F,
                        const double* const* pos, const double* const* vel, const double* const* vpos,
                        const double* const* cv, const double* const* cv1, const double* xb1, const double* vb1,
                        const double* Cb1, const double* Fb1, const double* const* posb1,
                        const double* const* velb1, const double* const* vpb1, double* xb, double* vb, double* Cb,
                        double* Fb, double* const* posb, double* const* velb, double* const* vpb,
                        double* const* cvb, double* const* cvb1, double* mat_b, int svd_grad_mode) {
  return substep_bwd_impl<double>(sc, x, v, C, F, pos, vel, vpos, cv, cv1, xb1, vb1, Cb1, Fb1, posb1, velb1, vpb1,
                                  xb, vb, Cb, Fb, posb, velb, vpb, cvb, cvb1, mat_b, svd_grad_mode);
}

int orc_abi_version(void) { return 1; }

}  // extern "C"
