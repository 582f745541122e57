/* d2f.h — C ABI of the GB300 implicit-step library (libd2f.so).
 *
 * The library advances a batch of independent 2D scenes (the reference calls them
 * environments) by one implicit backward-Euler step each: the preconditioned nonlinear
 * CG solve of the reference's PNCG2DSolver.step_targets (implicit/solver.py:433-451),
 * with plane-strain Neo-Hookean P1 triangles, collider barriers with lagged friction, IPC
 * point-edge contact between bodies, affine rigid bodies, the rigid-mode coarse space,
 * tendons and external forces.
 *
 * Ownership: every buffer is device memory owned by the caller (PyTorch tensors on the
 * Python side). The library borrows the pointers named in d2f_scene_desc for the life of
 * the handle and allocates nothing itself. All entry points are host functions; the
 * compute ones enqueue work on the stream given and return without synchronising.
 *
 * Errors: every entry point returns D2F_OK (0) or a negative D2F_E* code; d2f_last_error
 * gives the message of the last failure on the calling thread.
 */
#ifndef D2F_H
#define D2F_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define D2F_ABI_VERSION 7

/* status codes */
#define D2F_OK 0
#define D2F_EINVAL (-1)   /* bad argument, size or pointer */
#define D2F_ECUDA (-2)    /* a CUDA call failed */
#define D2F_ECAP (-3)     /* a scene's contact candidate list overflowed its capacity */
#define D2F_ENAN (-4)     /* a scene produced a non-finite step length */
#define D2F_ESPIN (-5)    /* a grid-wide barrier of the all-SM mode waited past its limit (2 s) */

/* blocks_per_scene: every SM on one scene at a time (a cooperative launch of one block per SM;
 * mixed precision; scenes taken in turn) */
#define D2F_ALL_SMS (-1)

/* precision modes */
#define D2F_FP64 0        /* every operation in FP64, as the reference runs */
#define D2F_MIXED 1       /* element, barrier and preconditioner arithmetic in FP32 */

/* Per-scene index ranges into the flat arrays (all scenes' data are contiguous, scene by
 * scene). One element per scene, device memory. Field order is part of the ABI. */
typedef struct d2f_seg {
    int32_t node0, nn;      /* nodes */
    int32_t tri0, nt;       /* triangles */
    int32_t bnd0, nb;       /* boundary nodes (slots into bnd[]) */
    int32_t edge0, ne;      /* boundary edges (IPC) */
    int32_t cand0, ncap;    /* contact-candidate list: first slot, capacity */
    int32_t bc0, nbc;       /* kinematic nodes (slots into bc_idx[]) */
    int32_t aff0, naff;     /* affine regions */
    int32_t affn0, naffn;   /* affine region node entries */
    int32_t rig0, nrig;     /* rigid-mode pieces */
    int32_t rign0, nrign;   /* rigid-mode piece node entries */
    int32_t ten0, nten;     /* tendons */
    int32_t tent0, ntent;   /* tendon eyelet entries */
    int32_t sp0, nsp;       /* springs and pins */
    int32_t pe0, npe;       /* pressure boundary edges */
} d2f_seg;

/* Everything one solver needs. Pointers are device pointers unless noted; arrays of
 * "real" are double in D2F_FP64 mode and float in D2F_MIXED mode. Field order is part
 * of the ABI. */
typedef struct d2f_scene_desc {
    int32_t abi_version;         /* = D2F_ABI_VERSION */
    int32_t precision;           /* D2F_FP64 | D2F_MIXED */
    int32_t n_scenes, N, T, Nb, Ne, n_bc, n_col;
    int32_t n_aff, n_affn, n_rig, n_rign, n_ten, n_tent, cand_total;
    int32_t max_nb;              /* largest boundary-node count of one scene (IPC rebuild buffer) */
    const d2f_seg *segs;         /* n_scenes */
    /* node state */
    double *x, *v, *xn, *xhat;   /* N x 2 */
    double *xu;                  /* 2 N + 6 n_aff doubles: the line search's saved state (positions,
                                    then affine coordinates; NULL without it) */
    const double *xrest;         /* N x 2: rest positions (mixed precision; else NULL) */
    void *grad, *grad_prev, *p, *diagH, *diag_el; /* N x 2 real */
    const double *mass;          /* N */
    const uint8_t *free_mask;    /* N: bit 0 = x free, bit 1 = y free */
    const double *fext;          /* N x 2, or NULL: the ExternalForce term (gravity folded in) */
    const int32_t *inc_ptr;      /* N + 1: CSR of the triangles at each node */
    const int32_t *inc;          /* 3 T: 3 * triangle + corner, ascending triangle per node */
    const int32_t *inc8;         /* N x 8: the first 8 entries of each node's inc list, -1 padded */
    const int32_t *node_bslot;   /* N: boundary slot of the node, or -1 */
    const int32_t *node_bc;      /* N: kinematic slot of the node, or -1 */
    const int32_t *node_aff;     /* N: affine node entry of the node, or -1 */
    const int32_t *node_rig;     /* N: rigid-mode piece node entry of the node, or -1 */
    /* triangles */
    const int32_t *tri;          /* T x 3 */
    const void *Bm;              /* T x 4 real: rest-shape inverse, row-major */
    const void *area, *mu, *lam; /* T real */
    const double *Dm;            /* T x 4: rest edge vectors X1-X0, X2-X0 (after any active-strain
                                    rest-shape change; mixed; else NULL) */
    void *escr;                  /* T x 12 real: per-corner gradient and diagonal */
    void *ecache;                /* T x 9 real: F^-T, la log J - mu, edge vectors */
    void *mscr;                  /* mixed precision: per-step scratch of d2f_mixed_scratch_bytes() bytes; else NULL */
    /* boundary nodes and colliders */
    const int32_t *bnd;          /* Nb: node of each boundary slot */
    const double *colliders;     /* n_col x 8: kind, cx, cy, rx, ry, rref, r, mu */
    const double *col_mu_env;    /* n_scenes x n_col per-scene collider friction, or NULL */
    /* kinematic nodes */
    const int32_t *bc_idx;       /* n_bc */
    const double *bc_target;     /* n_bc x 2 */
    /* IPC contact between bodies (Ne > 0 enables it) */
    const int32_t *ea, *eb, *ela, *elb; /* Ne */
    const double *ca, *cb;       /* Ne */
    const int32_t *excl_ptr, *excl_idx; /* CSR over boundary slots: excluded local slots, sorted */
    const double *mu_node;       /* N, or NULL: per-body friction (harmonic mean per pair) */
    int32_t *cand;               /* cand_total: packed (edge local << 16 | slot local), sorted */
    double *cand_tr;             /* cand_total x 2: per-pair ACCD profile of the current pass */
    double *xref;                /* Nb x 2: positions the candidate list was built at */
    /* tendons */
    const int32_t *t_node, *t_prv, *t_nxt, *t_tid; /* n_tent (prv/nxt/tid are global) */
    const double *t_stiff, *t_L0, *t_Tcmd;          /* n_ten */
    double *t_state;             /* n_ten x 4: L, dL, tau, keff */
    /* affine bodies */
    const int32_t *a_node, *a_grp; /* n_affn (grp global) */
    const double *a_w;           /* n_affn x 3 */
    const double *a_Mu, *a_La;   /* n_aff */
    double *a_q, *a_pq, *a_gq, *a_gq_prev, *a_zq; /* n_aff x 6 */
    double *a_H;                 /* n_aff x 18: J^T D J blocks (x, y) */
    /* rigid-mode coarse space */
    const int32_t *r_node, *r_grp; /* n_rign (grp global) */
    double *r_acc, *r_zq;        /* n_rig x 3 */
    /* per-scene outputs */
    int32_t *iters, *active, *status; /* n_scenes */
    int32_t *work;               /* 4 ints of scratch (the scene queue head) */
    /* parameters */
    double dt, drag, dhat, kappa, epsv, eps, tol_x, near_factor, alpha_max, area_shrink;
    double ccd_eta, cg_guard, gtol;
    double ipc_mu, ipc_dhat, ipc_kappa, reach, gap, bc_floor, skin;
    int32_t iter_max, conv_check, friction, per_body;
    int32_t threads;             /* threads per scene block: 32, 64, 128 or 256 (0: 256 for at most two
                                    scenes per SM, else 128) */
    int32_t blocks_per_sm;       /* resident scene blocks per SM the register budget targets
                                    (0: the library's default for that width) */
    /* backtracking energy line search (PNCG2DSolver line_search, solver.py:397-425; with
       affine bodies AffineBodies.save/trial, affine.py:383-389): both precisions, the energy
       summed in FP64 per scene; needs xu */
    double ls_tol;               /* accept while E <= E0 + ls_tol (|E0| + 1) */
    int32_t line_search;         /* 0 off, 1 on */
    int32_t n_backtrack;         /* halvings tried per iteration */
    int32_t blocks_per_scene;    /* mixed precision: thread blocks working on one scene, as one
                                    cluster of 512-thread blocks: 1, 8, 12 or 16 (0: a cluster of
                                    16, 12 or 8, whichever finishes the batch first, when the
                                    batch has fewer scenes than SMs and at least 16384 nodes per
                                    scene; else 1), or D2F_ALL_SMS: one 512-thread block per SM,
                                    all on one scene at a time (a cooperative launch; the library's
                                    choice where the device cannot co-schedule them) */
    const int32_t *a_ptr;        /* n_aff + 1: affine body b owns entries a_ptr[b] .. a_ptr[b+1]-1 of
                                    a_node / a_grp / a_w (required with affine bodies) */
    /* springs and pins (Springs, implicit/actuation.py:381-476): E = k/2 (|x_a - x_b| - L0)^2,
       x_b the node sp_b, or the world point sp_anchor where sp_b = -1 */
    int32_t n_sp;
    const int32_t *sp_a, *sp_b;  /* n_sp (global node ids) */
    const double *sp_k, *sp_L0;  /* n_sp: stiffness [Pa], rest length [m] */
    const double *sp_anchor;     /* n_sp x 2 */
    /* pressure boundaries (Pressure, implicit/actuation.py:80-152): E = -p A, A the shoelace
       area inside a chamber's directed edges (fluid on the left) */
    int32_t n_pe, n_ch;
    const int32_t *pe_a, *pe_b, *pe_ch; /* n_pe: edge start / end node, chamber (global ids) */
    const double *ch_p;          /* n_ch: gauge pressure [Pa] */
    const double *ch_ref;        /* n_ch x 2: the shoelace sum's reference point (energy) */
    double *energy_out;          /* NULL for a step; set by d2f_energy only */
} d2f_scene_desc;

typedef struct d2f_solver d2f_solver;

/* Library ABI version (D2F_ABI_VERSION of the build). */
int32_t d2f_abi_version(void);

/* Validate `desc` and create a solver handle that borrows its pointers.
 * Replaces the reference's PNCG2DSolver.__init__ (implicit/solver.py:97-226) together
 * with ImplicitIntegrator._build (implicit/integrator.py:252-311): the Python side builds
 * the scene arrays, this call binds them. */
int32_t d2f_create(const d2f_scene_desc *desc, d2f_solver **out);

/* One implicit step of every scene, enqueued on `stream` (a cudaStream_t; NULL = legacy
 * default stream). Kinematic targets are read from desc->bc_target.
 * Replaces PNCG2DSolver.step_targets (implicit/solver.py:433-451), as called by
 * ImplicitIntegrator.simulate (implicit/integrator.py:81-86). */
int32_t d2f_step(d2f_solver *s, void *stream);

/* Change the step size (and everything derived from it).
 * Replaces PNCG2DSolver.set_dt (implicit/solver.py:228-233). */
int32_t d2f_set_dt(d2f_solver *s, double dt, int32_t iter_max);

/* Per-scene status of the last step: iterations, still-active flag and error code are in
 * desc->iters / desc->active / desc->status (device). This call copies them to host
 * arrays of n_scenes entries (any may be NULL) after synchronising `stream`.
 * Replaces ImplicitIntegrator.stats (implicit/integrator.py:124-135). */
int32_t d2f_stats(d2f_solver *s, void *stream, int32_t *iters, int32_t *active, int32_t *status);

/* Release the handle (the caller's buffers are untouched). */
int32_t d2f_destroy(d2f_solver *s);

/* Message of the last error on this thread ("" if none). */
const char *d2f_last_error(void);

/* Bytes of the mixed-precision per-step scratch (d2f_scene_desc.mscr) for a batch of N
 * nodes, T triangles, Nb boundary nodes, n_col colliders and n_rig rigid-mode pieces. */
size_t d2f_mixed_scratch_bytes(int32_t N, int32_t T, int32_t Nb, int32_t n_col, int32_t n_rig);

/* Number of kernels d2f_step launches per call (for launch accounting). */
int32_t d2f_kernels_per_step(const d2f_solver *s);

/* Strain and stress of every triangle at positions x (core/fields.py: element_field; the
 * read-outs Model.element_strain / element_stress, sim_model.py:625-642), FP64 device arrays:
 * tri (T x 3), Bm (T x 4 row-major rest-shape inverse), mu, lam (T), x (N x 2). Outputs (T,
 * NULL to skip): the von Mises Green-Lagrange strain, its signed in-plane principal value,
 * the von Mises Neo-Hookean Cauchy stress, its signed principal value. One launch on stream. */
int32_t d2f_element_fields(int32_t T, const int32_t *tri, const double *Bm, const double *mu, const double *lam,
                           const double *x, double *strain_vm, double *strain_signed, double *stress_vm,
                           double *stress_signed, void *stream);

/* Contact read-outs at the solver's current x, with the last step's slip from x_n
 * (PNCG2DSolver.contact_force / collider_force, implicit/solver.py:553-612). what 0: the force
 * contact exerts on every node into out (N x 2 doubles; zeroed first): flags 1 colliders'
 * barrier, 2 contact between bodies, 4 friction; every DOF. what 1: the reaction on collider
 * `collider` (all of them when < 0) per scene into out (n_scenes x 2), flag 4 adds friction. */
int32_t d2f_contact_force(d2f_solver *s, int32_t what, int32_t collider, int32_t flags, double *out, void *stream);

/* Total energy of every scene at the solver's current state (PNCG2DSolver.energy,
 * implicit/solver.py:453-502): inertia against the last step's prediction, elastic,
 * collider barriers and lagged friction, external force, affine bodies, IPC, springs,
 * pressure, tendons; into out (n_scenes doubles, device). Moves nothing. FP64 solvers. */
int32_t d2f_energy(d2f_solver *s, double *out, void *stream);

/* The launch shape d2f_step uses: blocks launched, threads per block, blocks per scene (1: a
 * block per scene; 8, 12 or 16: one cluster per scene). Null outputs are skipped. */
int32_t d2f_launch_shape(const d2f_solver *s, int32_t *blocks, int32_t *threads, int32_t *blocks_per_scene);

/* Size of the library's static device scratch used by d2f_step_noalloc (16 MiB). */
#define D2F_NOALLOC_SCRATCH_BYTES (16u << 20)

/* One implicit step of every scene, like d2f_step, for callers that cannot allocate
 * device memory (a host that forbids cudaMalloc after start-up, a plugin handed plain
 * pointers by its host). No handle and no allocation: the caller passes the descriptor
 * with its inputs and outputs; the scratch fields (escr, ecache, mscr, cand, cand_tr, xref, work) are
 * ignored and taken from a static device array of D2F_NOALLOC_SCRATCH_BYTES that every
 * GPU loading the library holds until exit. A batch needing more scratch than that is
 * refused with D2F_EINVAL and a message. The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress); make that first call before any stream capture.
 * The address is kept for the life of the process: after cudaDeviceReset on a device, do
 * not call this entry point again on it. Every call shares the array and keeps the last
 * call's contents (the queue head is cleared, the candidate lists are rebuilt at each step
 * start): calls that overlap on the GPU race — serialise them.
 * No counterpart in the reference: its solver always owns its own buffers. */
int32_t d2f_step_noalloc(const d2f_scene_desc *desc, void *stream);

/* ---- adjoint of a converged step (FP64 solvers only) ----
 *
 * Solve, per scene, the transposed linearised step system at the converged positions x_lin
 * (N x 2, device):
 *     (M + h^2 (K_elastic + K_collider + K_tendon + K_spring + K_pressure + K_ipc)) lam = rhs
 * on the free DOFs, with the collider contact gate and the set of active IPC barrier terms
 * frozen at x_lin and friction left out, by preconditioned CG run on the device, one thread
 * block per scene. Affine bodies enter in their reduced coordinates: the system is
 * S^T H S + h^2 K_A with x = J q on a body's nodes and K_A its exact elastic block at its A
 * (recovered from x_lin), preconditioned per body by the inverse of its 6x6 block; lam is
 * J lam_q on the body's nodes. `rhs` (N x 2) is read on the free DOFs only; `lam` (N x 2)
 * gets the solution, zero on the kinematic DOFs; with warm_start != 0 the CG starts from the
 * `lam` passed in (e.g. the next step's adjoint, which a step's adjoint is close to), else
 * from zero. `work` is d2f_adjoint_work_doubles(s) doubles of scratch. `tension` (n_ten,
 * device, or NULL = desc->t_Tcmd) is the tension of each tension-controlled tendon at this
 * step. A scene stops when |r| <= rtol |rhs| or after max_iter iterations; per scene,
 * `iters` (device, n_scenes) gets the iterations and `status` (device, n_scenes) 0
 * (converged), 1 (max_iter reached), D2F_ENAN (the operator was not positive along a search
 * direction) or D2F_ECAP (more active IPC pairs than the scene's candidate capacity). The
 * handle's per-triangle scratch (escr, ecache) is overwritten: call between steps, not
 * during one. Refused (D2F_EINVAL) for mixed-precision solvers.
 * Replaces AdjointPNCG2D.adjoint_solve (implicit/adjoint.py:339-369), whose MINRES runs on
 * the host and crosses to the device twice per matrix-vector product; the reference refuses
 * IPC contact and affine bodies (:372-385). */
/* Doubles of scratch d2f_adjoint_solve needs for this solver: 12 N, plus 24 per IPC
 * candidate slot, plus 112 per affine body. */
int64_t d2f_adjoint_work_doubles(const d2f_solver *s);
int32_t d2f_adjoint_solve(d2f_solver *s, const double *x_lin, const double *rhs, double *lam, double *work,
                          const double *tension, double rtol, int32_t max_iter, int32_t warm_start, int32_t *iters,
                          int32_t *status, void *stream);

/* Vector-Jacobian products of one step's residual, accumulated for a solved lam:
 *   dscale[t]   += -h^2 lam . f_t(x_lin)    (f_t: triangle t's elastic force at its current
 *                                            mu, lam; the derivative with respect to a common
 *                                            scale of the triangle's two moduli)
 *   dtension[k]  = -h^2 lam . dL_k/dx       (L_k: length of tendon k; NULL to skip)
 * Replaces AdjointPNCG2D.drho (implicit/adjoint.py:277-283, drho_kernel :164-178), which
 * returns the same product pre-multiplied by the density map's (1 - Emin). */
/* dL/dp += the product of lam (from d2f_adjoint_solve at x_lin) with the derivative of the
 * step's residual with respect to each chamber's pressure (n_ch doubles, atomics). The
 * pressure and spring terms are in d2f_adjoint_solve's operator. */
int32_t d2f_adjoint_vjp_pressure(d2f_solver *s, const double *x_lin, const double *lam, double *dpressure,
                                 void *stream);

int32_t d2f_adjoint_vjp(d2f_solver *s, const double *x_lin, const double *lam, double *dscale, double *dtension,
                        void *stream);

#ifdef __cplusplus
}
#endif
#endif /* D2F_H */
