/*
 * difftactile_gb300 — C ABI of the GB300-native DiffTactile simulation substep.
 *
 * One substep couples an MLS-MPM object (quadratic B-spline P2G -> grid update with walls and
 * penalty contact -> G2P, deformation-gradient update with optional von-Mises return mapping)
 * with FEM tetrahedral elastomer sensors (tet elastic forces, explicit integration with a
 * kinematically driven base layer) through a grid-node <-> surface-triangle penalty/friction
 * contact.  Every forward kernel has a hand-written adjoint.
 *
 * Ownership: the library allocates nothing (except where an entry point says otherwise).  The
 * caller allocates every device buffer named in dt_world, fills the static tables, and passes
 * a host pointer to the dt_world descriptor to each call.  All calls are asynchronous on the
 * given stream and return DT_OK or a negative DT_ERR_* code for argument errors detected on the
 * host.  Errors found on the device (a particle that left the grid's safe band, a non-finite
 * value) are OR-ed into err[0] as DT_DEVERR_* bits; read err[0] after the stream completes.
 *
 * Reference interfaces replaced (paths inside the DiffTactile project):
 *   MPMObj.compute_new_F/svd/p2g         difftactile/object_model/mpm_elastic.py:135-208,
 *                                        difftactile/object_model/mpm_plastic.py:181-256,
 *                                        difftactile/object_model/multi_obj.py:228-252
 *   MPMObj.check_grid_occupy/grid_op     difftactile/object_model/mpm_elastic.py:211-240
 *   MPMObj.g2p                           difftactile/object_model/mpm_elastic.py:244-260
 *   FEMDomeSensor.update/update2         difftactile/sensor_model/fem_sensor.py:409-457,
 *                                        difftactile/sensor_model/gripper_fem.py:375-418
 *   Contact.check_collision/collision    difftactile/tasks/grasp_plastic.py:270-299 with
 *                                        find_closest/find_sdf fem_sensor.py:344-394 and
 *                                        calculate_contact_force grasp_plastic.py:205-216
 *   Contact.update / update_grad         difftactile/tasks/grasp_plastic.py:151-178
 *   MPMObj.svd_grad                      difftactile/object_model/mpm_elastic.py:145-173
 *   Contact.clamp_grid                   difftactile/tasks/grasp_plastic.py:192-202
 *
 * Layouts (all float buffers are IEEE fp32, all index buffers int32):
 *   particle state tape  p_state[n_frames][6][n_particles][4]: plane k of frame f holds floats
 *                        4k..4k+3 of the 24-float record
 *                        [x0 x1 x2 v0 | v1 v2 C00 C01 | C02 C10 C11 C12 | C20 C21 C22 F00 |
 *                         F01 F02 F10 F11 | F12 F20 F21 F22]   (C, F row-major)
 *   particle adjoint     p_adj[2][6][n_particles][4], same record layout, double-buffered.
 *   grid                 flat over all envs in 4x4x4-node blocks: node (i,j,k) of env e lives at
 *                        e.node_off + 64*((bi*nb1 + bj)*nb2 + bk) + 16*(i&3) + 4*(j&3) + (k&3),
 *                        bi = i>>2 ...; g_acc = (momentum.xyz, mass), g_vout = (v.xyz, 0).
 *   FEM vertex frames    v_pos/v_vel/v_velmid/v_ext/v_vpos/v_cv [n_frames][n_verts][4] (xyz, 0).
 */
#ifndef DIFFTACTILE_GB300_H
#define DIFFTACTILE_GB300_H

#include <stddef.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DT_ABI_VERSION 8

#define DT_OK 0
#define DT_ERR_ARG (-1)        /* null pointer, bad size or frame index */
#define DT_ERR_LAUNCH (-2)     /* a kernel launch failed (cudaGetLastError) */
#define DT_ERR_CAPACITY (-3)   /* a size exceeds a compiled or documented maximum */

/* device error bits, OR-ed into err[0] */
#define DT_DEVERR_PARTICLE_OOB 1   /* a particle's B-spline stencil left the grid: it was skipped */
#define DT_DEVERR_TAPE_FULL    2   /* more active grid blocks than tape_blocks in one frame */
#define DT_DEVERR_NONFINITE    4   /* NaN/Inf met in a grid node, a particle or a sensor vertex */
#define DT_DEVERR_ROPE_ITERS   8   /* a rope's iters exceeds max_rope_iters (or r_work is NULL): its
                                      adjoint was skipped */

#define DT_MAX_SENSORS_PER_ENV 4
#define DT_BLOCK_NODES 64

/* material model ids */
#define DT_MODEL_COROTATED 0   /* fixed-corotated, J = det(Sigma)         mpm_elastic.py:183-187 */
#define DT_MODEL_VON_MISES 1   /* fixed-corotated + von-Mises return map  mpm_plastic.py:151-166,228-235 */
#define DT_MODEL_NEOHOOKEAN 2  /* Kirchhoff stress mu(FF^T - I) + lam log(J) I                 */

/* grid boundary conditions */
#define DT_BC_SLIP_WALLS 0     /* reference: zero the inward normal velocity within `bound` nodes */
#define DT_BC_STICKY_FLOOR 1   /* slip walls, but all velocity zeroed on the floor band (j < bound) */

typedef struct dt_env {
  int p_begin, p_end;   /* particle range of this environment's object */
  int node_off;         /* first node of this env's grid in the flat grid arrays (multiple of 64) */
  int blk_off;          /* first block of this env */
  int nb[3];            /* blocks per axis */
  int n[3];             /* grid nodes per axis (n_grid in the reference); n[d] <= 4*nb[d] */
  int bound;            /* wall band in nodes (reference: 3) */
  int bc;               /* DT_BC_* */
  int s_begin, s_end;   /* sensors in contact with this env's object */
  float dx, inv_dx;     /* grid spacing and its inverse (each rounded from double) */
  float p_mass;         /* particle mass */
  float stress_k;       /* -dt * p_vol * 4 * inv_dx^2 (rounded from double) */
  float eps;            /* grid mass epsilon (1e-5) */
  float g2p_k;          /* 4 * inv_dx */
  float dt_g[3];        /* dt * gravity */
  float kn, kd, kt, mu_t;  /* contact: normal stiffness, normal damping, tangential stiffness, friction */
  float pad_;
} dt_env;

typedef struct dt_sensor {
  int v_off, nv;        /* vertex range in the flat FEM vertex arrays */
  int t_off, nt;        /* tet range */
  int f_off, nf;        /* surface triangle range */
  int env;              /* environment whose object this sensor touches */
  int carry;            /* 1: vel[f+1] += cv[f+1]-cv[f] (gripper_fem.py:415), 0: fem_sensor.py:454 */
  float dt_over_m;      /* dt / node mass */
  float mu, lam, alpha; /* elastomer Lame parameters, alpha = 1 + 0.75 mu/lam */
  float out_dir[3];     /* rot_h @ (0,1,0): orients surface normals (fem_sensor.py:340,370) */
  int model;            /* DT_FEM_*: elastomer force model */
} dt_sensor;

/* elastomer force models of the FEM sensors */
#define DT_FEM_REFERENCE 0          /* the reference's: P = mu (1 - 1/(I_C + 1)) F + lam (J - alpha) dJ/dF, current
                                       volume (fem_sensor.py:424-435) */
#define DT_FEM_LINEAR_COROTATED 1   /* P = 2 mu (F - R) + lam tr(R^T F - I) R, R the polar rotation of F, rest
                                       volume */

typedef struct dt_material {
  float mu, lam, yield_stress;
  int model;            /* DT_MODEL_* */
} dt_material;

/* PBD rope (PBDRope, PBD_rope.py:16-99) and its contact with the sensors of its environment
 * (cable_straightening.py:212-224, 288-319).  Node 0 is pinned at pin. */
typedef struct dt_rope {
  int p_off, n;         /* particle range in the flat rope arrays */
  int env;              /* environment whose sensors the rope touches (s_begin..s_end) */
  int blk_off;          /* first CTA of this rope in the rope-contact launches (64 particles per CTA) */
  float mass, inv_m;    /* p_mass = rho 4/3 pi rad^3 and its inverse */
  float rad;            /* particle radius = contact offset */
  float rest, bend;     /* stretch and bending rest lengths */
  float alpha_s, alpha_b;   /* compliance / dt^2 */
  float relax_s, relax_b;   /* relaxation factors */
  float table_h, friction;  /* floor height, tangential velocity factor on the floor */
  float dt_g[3];        /* dt * gravity */
  float pin[3];         /* position of node 0 */
  float kn, kd, kt, mu_t;   /* rope-sensor contact (no clamp of the normal approach speed) */
  int iters;            /* stretch + bending pass pairs per substep (<= 1: one, as PBDRope.update); the
                           adjoint of more than one needs dt_world.r_work */
} dt_rope;

/* World descriptor: host struct holding device pointers and sizes. */
typedef struct dt_world {
  /* ---- static tables (device) ---- */
  const dt_env* envs;            /* [n_envs] */
  const dt_sensor* sensors;      /* [n_sensors] */
  const dt_material* materials;  /* [n_materials] */
  const int* p_env;              /* [n_particles] env of each particle, non-decreasing */
  const int* p_mat;              /* [n_particles] material index of each particle */
  const int* blk_env;            /* [n_blocks] env of each block */
  const int* tets;               /* [n_tets][4] global vertex ids */
  const float* tet_B;            /* [n_tets][12] rest-shape inverse, 3 rows padded to 4 */
  const int* tet_sensor;         /* [n_tets] */
  const int* tris;               /* [n_tris][4] (a, b, c, sensor) global vertex ids */
  const int* tri_perm;           /* [n_tris] contact-search order: position -> triangle (global index),
                                    spatially compact within each sensor; NULL = identity */
  const int* v_layer;            /* [n_verts] layer id; layer 0 is kinematically driven */
  const int* v_sensor;           /* [n_verts] */
  /* ---- particle state ---- */
  float* p_state;                /* [n_frames][6][n_particles][4] */
  float* p_adj;                  /* [2][6][n_particles][4] */
  /* ---- grid working arrays (zero-invariant where noted) ---- */
  float* g_acc;                  /* [n_nodes][4] P2G accumulator, zero between substeps */
  float* g_vout;                 /* [n_nodes][4] */
  float* g_adj_vout;             /* [n_nodes][4] G2P adjoint accumulator, zero between substeps */
  float* g_adj_acc;              /* [n_nodes][4] */
  int* blk_flag;                 /* [n_blocks] zero between substeps */
  /* ---- per-frame grid tape ---- */
  int* tape_blist;               /* [n_frames][n_blocks] active block ids */
  int* tape_bcount;              /* [n_frames] */
  float* tape_acc;               /* [n_frames][tape_blocks*64][4] */
  float* tape_vout;              /* [n_frames][tape_blocks*64][4] */
  int* tape_cidx;                /* [n_frames][tape_blocks*64][4] argmin triangle per env sensor */
  /* ---- FEM frames ---- */
  float* v_pos;                  /* [n_frames][n_verts][4] */
  float* v_vel;                  /* [n_frames][n_verts][4] */
  float* v_velmid;               /* [n_frames][n_verts][4] vel after elastic forces */
  float* v_ext;                  /* [n_frames][n_verts][4] contact force accumulator */
  float* v_vpos;                 /* [n_frames][n_verts][4] virtual (kinematic) position */
  float* v_cv;                   /* [n_frames][n_verts][4] control velocity per frame */
  float* tri_cent;               /* [n_tris][4] working: centroids of the current frame */
  /* ---- FEM adjoints ---- */
  float* v_adj_pos;              /* [2][n_verts][4] */
  float* v_adj_vel;              /* [2][n_verts][4] */
  float* v_adj_vpos;             /* [2][n_verts][4] */
  float* v_adj_velmid;           /* [n_verts][4] */
  float* v_adj_ext;              /* [n_verts][4] contact-force adjoint of the frame in the backward sweep;
                                    zero between backward substeps (see dt_contact_force_bwd) */
  float* v_adj_cv;               /* [n_frames][n_verts][4] */
  float* mat_adj;                /* [n_materials][4] (d/dmu, d/dlam, 0, 0) accumulated */
  int* err;                      /* [4] device error word */
  /* ---- sizes ---- */
  int n_envs, n_particles, n_sensors, n_materials;
  int n_verts, n_tets, n_tris;
  int n_nodes, n_blocks, n_frames, tape_blocks;
  float dt;
  float grad_clip;               /* backward clamp of grid-mass and sensor grads; 0 disables */
  int svd_sweeps;                /* cyclic Jacobi sweeps of the 3x3 SVD (4 is enough for fp32) */
  int svd_grad_mode;             /* DT_SVDGRAD_* */
  int max_sensor_tris;           /* largest nf over the sensors (sizes the contact search's staging) */
  int scatter_mode;              /* DT_SCATTER_*: how P2G and the G2P adjoint accumulate into the grid */
  /* ---- PBD ropes (may be empty) ---- */
  const dt_rope* ropes;          /* [n_ropes] */
  float* r_state;                /* [n_frames][2][n_rope_particles][4]: (pos.xyz, travel), (vel.xyz, 0) */
  float* r_ext;                  /* [n_frames][n_rope_particles][4]: contact force * dt summed, contact flag */
  int* r_cidx;                   /* [n_frames][n_rope_particles][4] argmin triangle per env sensor */
  float* r_adj;                  /* [2][2][n_rope_particles][4] adjoint of r_state, double-buffered */
  float* r_extb;                 /* [n_rope_particles][4] working: adjoint of r_ext of the current frame */
  int n_ropes, n_rope_particles;
  int rope_blocks;               /* CTAs of the rope-contact launches (sum of ceil(n / 64)) */
  int max_rope_n;                /* largest n over the ropes (sizes the rope solver's shared memory) */
  /* ---- optional SVD tape ---- */
  float* p_svd;                  /* [n_frames][6][n_particles][4]: U, V, sigma of F_new per frame, written
                                    by the forward, read by the adjoint instead of recomputing; NULL:
                                    the adjoint recomputes the SVD.  Planes (U00 U01 U02 U10)
                                    (U11 U12 U20 U21) (U22 V00 V01 V02) (V10 V11 V12 V20) (V21 V22 s0 s1)
                                    (s2 y 0 0), y = 1 where the von Mises return map yielded */
  /* ---- launch shape ---- */
  int p_block;                   /* threads per CTA of the particle / tet / vertex launches: 64, 128 or
                                    256 (any other value: 128; the TILE scatter always uses 128) */
  int scatter_depth;             /* WARP scatter: 1 or 2 caps the segmented reduction at that many
                                    shuffle steps (runs summed in windows of 2 or 4 lanes, one RED per
                                    window and node); any other value: the whole run, one RED per run
                                    and node */
  int contact_lanes;             /* lanes per active grid node in the contact search: 4 or 8 (any other
                                    value: 8) */
  int skip_tape;                 /* 1: the forward substeps write neither the grid tape (tape_acc,
                                    tape_vout, tape_cidx) nor the SVD tape, for a forward whose tape no
                                    backward reads (the first pass of a checkpointed rollout, whose
                                    backward sweep recomputes each step); the active-block lists are
                                    still kept.  0: both are written */
  /* ---- PBD rope solver iterations ---- */
  float* r_work;                 /* [2 * max_rope_iters][n_rope_particles][4] adjoint workspace: the input
                                    positions of every pass, recomputed by dt_rope_update_bwd; may be NULL
                                    when no rope has iters > 1 */
  int max_rope_iters;            /* largest iters over the ropes that r_work is sized for */
  /* ---- launch shape (ABI 5) ---- */
  int p_per_thread;              /* particles per thread of the particle-role launches (P2G, G2P and their
                                    adjoints): each CTA takes this many consecutive chunks of p_block
                                    particles; 1 or 2 (anything else means 1) */
  /* ---- concurrency (ABI 6) ---- */
  cudaStream_t aux_stream;       /* optional second stream of the same device: dt_substep_fwd runs the rope
                                    solver on it beside G2P, dt_substeps_bwd the solver's adjoint beside
                                    the P2G, G2P and grid adjoints (one CTA per rope leaves most SMs to
                                    the MPM stages).  Work forked onto it is joined back into the call's
                                    stream before the call returns.  NULL: everything on the call's
                                    stream. */
  cudaEvent_t aux_events[2];     /* fork and join events (cudaEventDisableTiming), required with aux_stream */
  /* ---- optional SVD tape of the linear corotated tets (ABI 7) ---- */
  float* t_svd;                  /* [n_frames][6][n_tets][4]: U, V, sigma of each DT_FEM_LINEAR_COROTATED
                                    tet's F per frame, in p_svd's plane layout, written by the forward,
                                    read by the tet adjoint instead of recomputing; NULL: recomputed */
  /* ---- launch shape (ABI 8) ---- */
  int scatter_depth_adj;         /* the G2P adjoint's WARP scatter: 1 or 2 caps its segmented reduction at
                                    that many shuffle steps, 3 sums whole runs; any other value (0): the
                                    P2G's scatter_depth.  The two scatters weigh shuffles against REDs
                                    differently (the adjoint has no block marking and fewer registers
                                    live across the stencil) */
} dt_world;

/* 27-node particle scatters: TILE gathers each CTA's stencil contributions per node in shared
 * memory and issues one vector RED per touched node; GLOBAL issues one 16-byte vector RED per
 * particle and node (L2 atomics); WARP first sums, over each run of consecutive lanes whose particles
 * share a base cell (particles are kept sorted by cell, so runs are long), with a segmented
 * shuffle reduction, then issues one RED per run and node; SMEM sums whole runs the same way, then
 * adds into a shared-memory tile of the grid around the CTA's particles (shared atomics) and flushes
 * the tile with one RED per touched node (falling back to WARP for a CTA whose particles' stencils
 * do not fit the tile).  scatter_depth caps the segmented reduction of WARP (SMEM ignores it). */
#define DT_SCATTER_TILE 0
#define DT_SCATTER_GLOBAL 1
#define DT_SCATTER_WARP 2
#define DT_SCATTER_SMEM 3

/* SVD adjoint of the rotation R = U V^T used by the corotated stress:
 * STABLE evaluates the reference formula's rotation term in the algebraically equal form
 * (M - M^T)_ij / (s_i + s_j), M = U^T dR V (exact in floating point near F = I);
 * REFERENCE evaluates mpm_elastic.py:158-173 literally, ff_ij = 1/clamp(s_j^2 - s_i^2, 1e-8). */
#define DT_SVDGRAD_STABLE 0
#define DT_SVDGRAD_REFERENCE 1

/* ---- introspection ---- */
int dt_abi_version(void);
size_t dt_sizeof_world(void);
size_t dt_sizeof_env(void);
size_t dt_sizeof_sensor(void);
size_t dt_sizeof_material(void);
size_t dt_sizeof_rope(void);

/* No counterpart in the reference.  Library-wide switch for programmatic dependent launch of the
 * substep kernels (default on: each kernel waits for its predecessor's completion in-kernel, so the
 * next launch overlaps the previous kernel's tail).  Returns the previous setting. */
int dt_set_pdl(int on);
/* The current setting of dt_set_pdl (1 on, 0 off). */
int dt_get_pdl(void);

/* No counterpart in the reference (Taichi raises Python exceptions).  The CUDA error behind the
 * last DT_ERR_LAUNCH returned to this host thread: writes "<name>: <description>" into buf (at most len bytes, NUL-terminated),
 * returns the cudaError_t code (0: none since the last call) and clears it.  Device-side problems
 * are reported through dt_world.err instead. */
int dt_last_error(char* buf, size_t len);

/* ---- step set-up ----
 * Clears the grid tape counters of every frame and prepares FEM frame 0 (velmid = vel, ext = 0).
 * Call once before the substeps of a control step (the reference calls Contact.reset(),
 * grasp_plastic.py:386). */
int dt_step_begin(const dt_world* w, cudaStream_t stream);

/* ---- forward substep f -> f+1 (replaces Contact.update(f), grasp_plastic.py:151-164) ----
 * Three launches: P2G + FEM tet forces + triangle centroids; grid update + contact; G2P + FEM
 * integration.  Requires 0 <= f < n_frames-1. */
int dt_substep_fwd(const dt_world* w, int f, cudaStream_t stream);

/* dt_substep_fwd split into its three launches (stage 0: P2G + FEM forces + centroids; 1: grid
 * update + contact; 2: G2P + FEM integration), for timing and for callers that interleave work. */
int dt_substep_fwd_stage(const dt_world* w, int f, int stage, cudaStream_t stream);

/* No counterpart in the reference.  dt_substep_fwd for callers that cannot allocate device memory
 * (their buffers live in memory another allocator owns, e.g. a framework's caching allocator or an
 * arena reserved at start-up under a fixed device-memory budget, so they may not call cudaMalloc).
 * The caller provides inputs and outputs as for dt_substep_fwd; the scratch (grid accumulator and
 * velocities, active-block flags and list, the frame's grid tape, triangle centroids) lives in one
 * static device array inside the library (~21 MB, held by every GPU that loads the library until the
 * process exits); w's scratch pointers are ignored and may be NULL.  Limits: n_nodes <= 64^3,
 * n_blocks <= 4096, n_tris <= 8192, else DT_ERR_CAPACITY.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before any stream capture.
 * The stream must belong to the current device (else DT_ERR_ARG).  The looked-up address is kept
 * for the life of the process: after cudaDeviceReset do not call this entry point again.
 * All calls share the array: calls that overlap on the GPU (other streams, other threads) race.
 * The grid tape written here is scratch, so dt_substep_bwd cannot follow this call; it allocates
 * nothing (no cudaMalloc, cudaFree or allocating library routine). */
int dt_substep_fwd_noalloc(const dt_world* w, int f, cudaStream_t stream);

/* ---- particle re-binning (keeps the particles sorted by cell over a rollout) ----
 * Replaces nothing in the reference, whose particle loops visit particles in their fixed order
 * (mpm_elastic.py:176-208); the scatter here merges same-cell runs of consecutive particles, which
 * the material's motion breaks up.  dt_rebin sorts the particles of frame f by the grid node of their
 * base cell (block-major node order; within a cell by current slot): src[j] = the current slot of
 * new slot j ([n_particles] device ints, written).  It permutes frame f's particle records and
 * p_mat (which must be the buffer w->p_mat points to: the material index follows its particle)
 * accordingly.  Every other frame, the SVD tape and the adjoints are not touched: re-bin only a frame
 * from which the next substeps start, with no tape frame before it still to be read in this order.
 * Requirements: the environments' node ranges (node_off) increase with the environment index, as
 * their particle ranges do (the sort then keeps every particle in its environment's range).
 * scratch: dt_rebin_scratch_bytes(w) bytes of device memory, 256-byte aligned.
 * Cells that hold more than 256 particles keep the (unordered) placement of the atomics. */
size_t dt_rebin_scratch_bytes(const dt_world* w);
int dt_rebin(const dt_world* w, int f, int* p_mat, int* src, void* scratch, cudaStream_t stream);
/* Applies the permutation src of a dt_rebin (inverse = 0: new[j] = old[src[j]]; inverse = 1:
 * old[src[j]] = new[j]) to p_mat and, for buf = 0 or 1, to the particle adjoint buffer p_adj[buf]
 * (buf = -1: p_mat only).  The backward sweep crosses a re-binning of frame f with inverse = 1 on the
 * buffer that holds frame f's adjoint: the adjoint then follows the order before the re-binning. */
int dt_rebin_permute(const dt_world* w, int buf, int inverse, int* p_mat, const int* src, void* scratch,
                     cudaStream_t stream);

/* The same substep split into the reference's per-object calls, for drop-in use of the
 * reference method sequence.  dt_substep_fwd(f) == p2g(f); fem_update(f); grid_op(f) (which
 * includes check_grid_occupy, check_collision and collision); rope_update(f); g2p(f);
 * fem_update2(f).  dt_substep_fwd_stage: stage 0 = p2g + fem_update, 1 = grid_op + rope_update,
 * 2 = g2p + fem_update2. */
int dt_p2g(const dt_world* w, int f, cudaStream_t stream);         /* mpm_elastic.py:135-208 */
int dt_fem_update(const dt_world* w, int f, cudaStream_t stream);  /* fem_sensor.py:409-440 */
int dt_grid_op(const dt_world* w, int f, cudaStream_t stream);     /* mpm_elastic.py:211-240 + grasp_plastic.py:270-299 */
int dt_g2p(const dt_world* w, int f, cudaStream_t stream);         /* mpm_elastic.py:244-260 */
int dt_fem_update2(const dt_world* w, int f, cudaStream_t stream); /* fem_sensor.py:444-457 */

/* Rope part of a substep (no-op without ropes): check_collision + collision of the rope particles
 * against their env's sensors (cable_straightening.py:288-319) and PBDRope.update(f)
 * (PBD_rope.py:112-180); writes r_state[f+1], r_ext[f], r_cidx[f] and adds the sensors' contact
 * forces to v_ext[f].  Runs after the sensors' elastic update and before their update2.  Shared
 * memory: 32 * max_rope_n bytes (DT_ERR_CAPACITY above 227 KB). */
int dt_rope_update(const dt_world* w, int f, cudaStream_t stream);
/* Adjoint of dt_rope_update (rope.update.grad, clamp_grid on the rope's grads, collision.grad;
 * cable_straightening.py:177-186): consumes r_adj[(f+1)&1] and v_adj_ext (after the FEM
 * update2 adjoint), writes r_adj[f&1], accumulates v_adj_velmid and v_adj_pos[f&1].  Shared memory:
 * 64 * max_rope_n bytes. */
int dt_rope_update_bwd(const dt_world* w, int f, cudaStream_t stream);

/* Copy frame `src` of the particle, FEM and rope state to frame `dst` (mpm_elastic.py:263-268,
 * fem_sensor.py:461-465, PBD_rope.py:182-187). */
int dt_copy_frame(const dt_world* w, int src, int dst, cudaStream_t stream);

/* ---- backward substep (replaces Contact.update_grad(f), grasp_plastic.py:167-178) ----
 * Consumes the adjoint of frame f+1 held in p_adj[(f+1)&1], v_adj_*[(f+1)&1] and produces the
 * adjoint of frame f in p_adj[f&1], v_adj_*[f&1]; accumulates v_adj_cv[f], v_adj_cv[f+1] and
 * mat_adj.  The forward tape of frame f (p_state[f], grid tape f, FEM frame f) must be intact. */
int dt_substep_bwd(const dt_world* w, int f, cudaStream_t stream);

/* dt_substep_bwd split into its four launches, the per-kernel .grad calls of update_grad
 * (grasp_plastic.py:167-178): stage 0 restores frame f's grid velocities from the tape; stage 1 is
 * fem.update2.grad + g2p.grad; stage 2 is grid_op.grad + clamp_grid + collision.grad (and
 * dt_rope_update_bwd); stage 3 is
 * fem.update.grad + p2g.grad + svd_grad + compute_new_F.grad.  Run stages 0..3 in order. */
int dt_substep_bwd_stage(const dt_world* w, int f, int stage, cudaStream_t stream);

/* dt_substep_bwd for f = f_hi - 1 down to f_lo in one call: the restore of frame f - 1 (stage 0) runs
 * inside stage 3 of frame f, one launch fewer per substep.  Same results as the sequence of
 * dt_substep_bwd calls. */
int dt_substeps_bwd(const dt_world* w, int f_hi, int f_lo, cudaStream_t stream);

/* Zero the adjoint buffers (p_adj, v_adj_*, mat_adj, g_adj_*, r_adj, r_extb) before a backward sweep. */
int dt_adj_clear(const dt_world* w, cudaStream_t stream);

/* ---- readouts ---- */
/* Per-env centre of mass of frame f: out[n_envs][4] (xyz, 0) (grasp_plastic.py:259-261). */
int dt_com(const dt_world* w, int f, float* out, cudaStream_t stream);
/* Adjoint of dt_com: adds adj_com[e]/count to x-adjoint of every particle of env e in p_adj[f&1]. */
int dt_com_bwd(const dt_world* w, int f, const float* adj_com, cudaStream_t stream);

/* ---- action input: pose control (fem_sensor.py:229-266, set_pose_control + set_control_vel) ----
 * cv_i = ((A vp_i + b) - vp_i) * inv_T for every vertex i of sensor s, vp = virtual positions of
 * frame f0, (A | b) = rows 0..2 of the step transform dtrans_h given as 12 device floats (row-major
 * 3x4), inv_T = 1 / (dt * substeps); written into frames [f0, f0 + nfr) of v_cv (one control step). */
int dt_pose_control_vel(const dt_world* w, int s, const float* Ab, float inv_T, int f0, int nfr,
                        cudaStream_t stream);
/* dt_pose_control_vel for every sensor in one launch: Ab [n_sensors][12] (device), sensor s's
 * transform in row s. */
int dt_pose_control_vel_all(const dt_world* w, const float* Ab, float inv_T, int f0, int nfr, cudaStream_t stream);
/* Adjoint: Ab_bar[12] (device) += sum_i cvb_i [vp_i, 1]^T inv_T and v_adj_vpos[f0&1] += (A - I)^T cvb_i
 * inv_T, with cvb_i the control-velocity adjoint summed over frames [f0, f0 + nfr) of v_adj_cv.  Those
 * entries of v_adj_cv are consumed (reset to zero), so consecutive control steps may share their
 * boundary frame: call it after the adjoint substeps of frames [f0, f0 + nfr - 1). */
int dt_pose_control_vel_bwd(const dt_world* w, int s, const float* Ab, float inv_T, float* Ab_bar, int f0, int nfr,
                            cudaStream_t stream);
/* dt_pose_control_vel_bwd for every sensor in one launch: Ab and Ab_bar are [n_sensors][12]. */
int dt_pose_control_vel_bwd_all(const dt_world* w, const float* Ab, float inv_T, float* Ab_bar, int f0, int nfr,
                                cudaStream_t stream);

/* ---- action input: gripper fingers (gripper_kinematics.py:196-216, fem_sensor1/2_set_control_vel) ----
 * For k < nfr: v_cv[f0 + k][i] = D[k][:, 0:3] src_i + D[k][:, 3] for every vertex i of sensor s, with
 * D [nfr][12] (device, row-major 3x4 per frame) and src [n_verts][4] (device) the points the
 * transforms act on (the sensors' rest positions, with T0^-1 folded into D). */
int dt_affine_control_vel(const dt_world* w, int s, const float* D, const float* src, int f0, int nfr,
                          cudaStream_t stream);
/* Adjoint: D_b[k] += sum_i v_adj_cv[f0 + k][i] [src_i, 1]^T (device, accumulated); the consumed
 * entries of v_adj_cv are reset to zero. */
int dt_affine_control_vel_bwd(const dt_world* w, int s, const float* src, int f0, int nfr, float* D_b,
                              cudaStream_t stream);

/* ---- shape-target (deform) loss (tasks/deform_loss.py:8-146) ----
 * Grids are [n_nodes] floats in the world's block layout (node_index of env e); nodes outside the
 * env's n^3 are ignored.  dt_grid_mass adds the mass-only P2G of env e's particles at frame f
 * (compute_grid_m_kernel, mpm_plastic.py:169-178; node i at i dx) into m (zero it first). */
int dt_grid_mass(const dt_world* w, int e, int f, float* m, cudaStream_t stream);
/* loss[0] (device, accumulated) += w_density sum |m - target| + w_sdf sum sdf m over env e's nodes
 * (compute_density_loss_kernel + compute_sdf_loss_kernel + sum_up_loss_kernel). */
int dt_deform_loss(const dt_world* w, int e, const float* m, const float* target, const float* sdf, float w_density,
                   float w_sdf, float* loss, cudaStream_t stream);
/* Adjoint: the x adjoint of frame f (p_adj[f&1], plane 0) += loss_bar d loss / d x through the mass
 * P2G (d|.|/d. = sign, 0 at 0). */
int dt_deform_loss_bwd(const dt_world* w, int e, int f, const float* m, const float* target, const float* sdf,
                       float w_density, float w_sdf, float loss_bar, cudaStream_t stream);
/* Target distance field (update_target / update_target_sdf): `passes` rounds (reference: 2 n_grid) of
 * nearest-seed propagation over offsets in [-3, 3)^3, seeds where target > 1e-4, distance
 * sqrt(|d|^2 + 1e-8), 1000 where unreached.  scratch: [2][n_nodes][4] floats. */
int dt_target_sdf(const dt_world* w, int e, const float* target, float* sdf, float* scratch, int passes,
                  cudaStream_t stream);

/* ---- rigid shape matching (multi_obj.py:309-340: compute_COM, compute_H) ----
 * Over env e's particles of material `mat` (the rigid part), between frames f and f+1:
 * out[0..2] = c0 = sum x_f / N, out[4..6] = c1 = sum x_{f+1} / N (N: all particles of the env, as the
 * reference), out[8..16] = H = sum (x_f - c0)(x_{f+1} - c1)^T row-major.  out: 20 device floats,
 * overwritten.  The 3x3 SVD of H, R = V U^T and the angle readout are left to the caller. */
int dt_rigid_match(const dt_world* w, int e, int mat, int f, float* out, cudaStream_t stream);
/* Adjoint for H_b (9 device floats, d loss / d H): part 0 adds d/dx_f to p_adj[f&1], part 1 adds
 * d/dx_{f+1} to p_adj[(f+1)&1] (call each while that frame's adjoint buffer is current).  out: the
 * forward's output; scratch: 8 device floats. */
int dt_rigid_match_bwd(const dt_world* w, int e, int mat, int f, int part, const float* out, const float* H_b,
                       float* scratch, cudaStream_t stream);

/* ---- contact-force readout (compute_contact_force, grasp_plastic.py:218-229) ----
 * out[0..2] (device, accumulated) += sum over sensor s's surface triangles of 1/6 of the contact
 * force v_ext[f] on each of the triangle's vertices. */
int dt_contact_force(const dt_world* w, int s, int f, float* out, cudaStream_t stream);
/* Adjoint: v_adj_ext += out_b[0..2] / 6 on each surface triangle's vertices.  v_adj_ext is the
 * adjoint of the contact forces of the frame whose backward substep runs next: call it for frame f
 * after dt_substep_bwd(f + 1) and before dt_substep_bwd(f). */
int dt_contact_force_bwd(const dt_world* w, int s, const float* out_b, cudaStream_t stream);

/* ---- marker readout (extract_markers, fem_sensor.py:161-187) ----
 * Fisheye camera of project_3d_2d (sensor_model/fisheye_model.py:12-30): the point is shifted by
 * `plane` along the optical axis z, theta = acos(z / |a|), omega = atan2(y, x + 1e-8) + pi,
 * pixel = m f theta (cos omega, sin omega) + (cx, cy).  The reference's defaults are
 * f = 8.627e-4, m = 173913.04, cx = 332, cy = 240, plane = 0.02. */
typedef struct dt_fisheye {
  float f, m, cx, cy, plane;
} dt_fisheye;
/* For marker m: pred[m] = sum_k wts[m K + k] proj(node), virt[m] the same of the virtual positions,
 * node = surf[idx[m K + k]] (local vertex ids of sensor s), proj = fisheye of (x, z, y) of
 * inv_trans (rows 0..2 of the 4x4 world-to-sensor transform, 12 device floats) applied to (p, 1).
 * pred, virt: [M][2] device. */
int dt_markers(const dt_world* w, int s, int f, const int* surf, const int* idx, const float* wts, int K, int M,
               const float* inv_trans, dt_fisheye cam, float* pred, float* virt, cudaStream_t stream);
/* Adjoint: v_adj_pos[f&1] and v_adj_vpos[f&1] += the position adjoints of pred_b, virt_b ([M][2]
 * device, either may be NULL); inv_trans_b[12] (device, may be NULL) += d/d inv_trans. */
int dt_markers_bwd(const dt_world* w, int s, int f, const int* surf, const int* idx, const float* wts, int K, int M,
                   const float* inv_trans, dt_fisheye cam, const float* pred_b, const float* virt_b,
                   float* inv_trans_b, cudaStream_t stream);

/* ---- tactile readout: marker-displacement loss (cf. grasp_plastic.py:241-256) ----
 * loss[0] (device) += sum over vertices i of sensor s with layer id `layer` of
 * |(pos_i - vpos_i) - target_i|^2 at frame f; target is [nv][4] device floats (xyz, pad). */
int dt_marker_loss(const dt_world* w, int s, int f, int layer, const float* target, float* loss,
                   cudaStream_t stream);
/* Adjoint: adds 2 loss_bar (disp - target) to v_adj_pos[f&1] and its negative to v_adj_vpos[f&1]. */
int dt_marker_loss_bwd(const dt_world* w, int s, int f, int layer, const float* target, float loss_bar,
                       cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* DIFFTACTILE_GB300_H */
