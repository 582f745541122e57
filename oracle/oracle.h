/* CPU FP64 oracle of the Diff_2D_FEM implicit step — TEST INFRASTRUCTURE.
 *
 * A plain-C restatement of the reference's PNCG-IPC solve (implicit/solver.py,
 * implicit/kernels.py, core/math.py, core/sdf.py, implicit/ipc_contact.py,
 * implicit/affine.py, implicit/actuation.py), executed the way the reference's Warp CPU
 * backend executes it: every kernel is a serial loop over its thread ids, every atomic is
 * applied in thread order, and the kernels run in the launch order of
 * PNCG2DSolver._iterate. It is the checker for the CUDA path and the timed CPU baseline;
 * the product never links it.
 *
 * The caller owns every buffer (numpy arrays passed by pointer); the oracle allocates
 * nothing but small per-call scratch.
 */
#ifndef D2F_ORACLE_H
#define D2F_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    /* sizes */
    int32_t N, T, B, Nb, n_bc, n_col;
    /* node state (N x 2, row-major) */
    double *x, *v, *xn, *xhat, *grad, *grad_prev, *p, *diagH, *x0buf;
    const double *mass;      /* N */
    double *free_;           /* N x 2 */
    const int32_t *node2env; /* N */
    /* elements */
    const int32_t *tri;      /* T x 3 */
    const double *Bm;        /* T x 2 x 2 row-major */
    const double *area, *mu, *lam;
    const int32_t *tri2env;
    /* boundary nodes */
    const int32_t *bnd, *b2e; /* Nb */
    /* kinematic nodes */
    const int32_t *bc_idx;   /* n_bc */
    double *bc_target;       /* n_bc x 2 */
    /* colliders: n_col x 8 (kind, cx, cy, rx, ry, rref, r, mu) */
    const double *colliders;
    /* per-env scalars (B) */
    double *gPg, *g_p, *g_Py, *y_p, *y_Py, *beta, *gTp, *pHp, *alpha, *p_inf, *clr_min,
           *dE, *dE0, *Ener, *Els_prev, *gn0;
    int32_t *active, *iters;
    /* parameters */
    double dt, h2, inv_dt, drag, dhat, kappa, epsv;
    double eps, tol_x, near_factor, alpha_max, area_shrink, ccd_eta, cg_guard, ls_tol, gtol;
    int32_t iter_max, conv_check, friction, line_search, n_bt;

    /* ---- ExternalForce term (has_ext) */
    int32_t has_ext;
    const double *fext;      /* N x 2 */

    /* ---- IPC contact between bodies (has_ipc) */
    int32_t has_ipc, Ne, per_body;
    const int32_t *ea, *eb, *ela, *elb, *e2env; /* Ne */
    const double *ca, *cb;                      /* Ne */
    const int32_t *bstart, *bpe;                /* B: first boundary slot, count per env */
    const int32_t *excl_ptr, *excl_idx;         /* CSR over boundary slots: excluded local slots, sorted */
    const double *mu_node;                      /* N (per_body) */
    double ipc_mu, ipc_dhat, ipc_kappa, reach, gap, bc_floor;
    double *q, *q_inf, *sweep_beta, *clr;       /* N x 2, B, B, B */
    int32_t pending;

    /* ---- Tendon term (n_tendon > 0) */
    int32_t n_tendon, n_tent;
    const int32_t *t_node, *t_prv, *t_nxt, *t_tid, *t2env;
    const double *t_stiff, *t_L0, *t_Tcmd;
    double *t_L, *t_dL, *t_tau, *t_keff;

    /* ---- AffineBodies mode (n_aff > 0) */
    int32_t n_aff, n_affn;
    const int32_t *a_node, *a_grp, *a_env;
    const double *a_w, *a_Mu, *a_La;            /* n_affn x 3, n_aff, n_aff */
    double *a_q, *a_q0, *a_pq, *a_gq, *a_gq_prev, *a_zq, *a_Hx, *a_Hy; /* n_aff x 6 / x 9 */

    /* ---- RigidModes mode (n_rig > 0) */
    int32_t n_rig, n_rign;
    const int32_t *r_node, *r_grp, *r_env;
    double *r_acc, *r_gq, *r_gq_prev, *r_zq, *r_Hc; /* n_rig x 3 / x 9 */
    double *diag_el;                                /* N x 2 */

    /* ---- Springs term (n_spring > 0): node b = -1 ties node a to the world point anchor */
    int32_t n_spring;
    const int32_t *sp_a, *sp_b, *sp2env;            /* n_spring */
    double *sp_k, *sp_L0, *sp_anchor;               /* n_spring, n_spring, n_spring x 2 */

    /* ---- Pressure term (n_pedge > 0): directed chamber edges, fluid on the left */
    int32_t n_pedge, n_chamber;
    const int32_t *pe_a, *pe_b, *pe_ch;             /* n_pedge */
    const int32_t *ch2env;                          /* n_chamber */
    double *ch_p, *ch_ref;                          /* n_chamber, n_chamber x 2 */
} d2o_solver;

/* One implicit step (PNCG2DSolver.step_targets), bc_target already set. */
int d2o_step(d2o_solver *s);
/* Kinematic sweep scratch is needed only when has_ipc && n_bc. */

/* Per-env total energy (PNCG2DSolver._energy_into) into s->Ener. */
void d2o_energy(d2o_solver *s, double *buf);
void d2o_ipc_energy(d2o_solver *s, double *buf);
/* One actuation term (0 Springs, 1 Pressure) alone at s->x: gradient, diagonal, curvature
   along s->p, energy per environment (test access). */
void d2o_term(d2o_solver *s, int which, double *E);
void d2o_affine_hessian(const double *A4, double Mu, double La, double h2, const double *Hx, const double *Hy,
                        double *H36);
void d2o_chol6_solve(const double *H36, const double *b, double *x);
/* A collider's level set at n points (x, y pairs) into d (test access). */
void d2o_sdf_full(int kind, double cx, double cy, double rx, double ry, double rref, const double *pts, int n,
                  double *d, double *g, double *H);
void d2o_sdf(int kind, double cx, double cy, double rx, double ry, double rref, const double *pts, int n,
             double *d);

/* Number of floating-point operations the element pass of one iteration would perform
 * is not counted here; see the Python side. */
#ifdef __cplusplus
}
#endif
#endif
