/* CPU FP64 oracle of the Diff_2D_FEM implicit step — TEST INFRASTRUCTURE (see oracle.h).
 *
 * Every function below restates one reference kernel or helper, named in its comment by
 * file:line of the reference. Expressions keep the reference's evaluation order (Python
 * left-to-right, which Warp's code generator preserves) so that, compiled without FMA
 * contraction (-ffp-contract=off), the oracle reproduces a serial execution of the
 * reference's own kernels bit for bit.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define BIG 1.0e30
#define LOG_EPS 1.0e-6

/* Test switch: 1 = every contact pair of a pass uses the step cap as it stood when the
 * pass began (instead of the reference's running value at the start of each edge). */
static int g_tc_fixed = 0;
void d2o_set_tc_fixed(int v) { g_tc_fixed = v; }

typedef struct { double x, y; } v2;
typedef struct { double a, b, c, d; } m2; /* row-major [[a, b], [c, d]] */

static inline v2 V(double x, double y) { v2 r = {x, y}; return r; }
static inline v2 add(v2 a, v2 b) { return V(a.x + b.x, a.y + b.y); }
static inline v2 sub(v2 a, v2 b) { return V(a.x - b.x, a.y - b.y); }
static inline v2 scl(double s, v2 a) { return V(s * a.x, s * a.y); }  /* s * v */
static inline v2 vsc(v2 a, double s) { return V(a.x * s, a.y * s); }  /* v * s */
static inline v2 vdiv(v2 a, double s) { return V(a.x / s, a.y / s); }
static inline v2 cw(v2 a, v2 b) { return V(a.x * b.x, a.y * b.y); }
static inline double dot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline double len(v2 a) { return sqrt(dot(a, a)); }
static inline double cross2(v2 a, v2 b) { return a.x * b.y - a.y * b.x; }  /* core/math.py:105-108 */
static inline double fmax_(double a, double b) { return a > b ? a : b; }
static inline double fmin_(double a, double b) { return a < b ? a : b; }
static inline double fabs_(double a) { return a >= 0 ? a : -a; }

static inline v2 ld(const double *a, int i) { return V(a[2 * i], a[2 * i + 1]); }
static inline void st(double *a, int i, v2 v) { a[2 * i] = v.x; a[2 * i + 1] = v.y; }
static inline void atomic_add2(double *a, int i, v2 v) { a[2 * i] = a[2 * i] + v.x; a[2 * i + 1] = a[2 * i + 1] + v.y; }
static inline void amin(double *a, int i, double v) { if (v < a[i]) a[i] = v; }
static inline void amax(double *a, int i, double v) { if (v > a[i]) a[i] = v; }

static inline m2 M(double a, double b, double c, double d) { m2 r = {a, b, c, d}; return r; }
static inline m2 mmul(m2 A, m2 B) {
    return M(A.a * B.a + A.b * B.c, A.a * B.b + A.b * B.d, A.c * B.a + A.d * B.c, A.c * B.b + A.d * B.d);
}
static inline v2 mvec(m2 A, v2 v) { return V(A.a * v.x + A.b * v.y, A.c * v.x + A.d * v.y); }
static inline m2 madd(m2 A, m2 B) { return M(A.a + B.a, A.b + B.b, A.c + B.c, A.d + B.d); }
static inline m2 msub(m2 A, m2 B) { return M(A.a - B.a, A.b - B.b, A.c - B.c, A.d - B.d); }
static inline m2 msc(double s, m2 A) { return M(s * A.a, s * A.b, s * A.c, s * A.d); }
static inline m2 mT(m2 A) { return M(A.a, A.c, A.b, A.d); }
static inline double ddot(m2 A, m2 B) { return A.a * B.a + A.b * B.b + A.c * B.c + A.d * B.d; }
static inline double det2(m2 A) { return A.a * A.d - A.c * A.b; }
static inline m2 inv2(m2 A) {
    double dt = det2(A);
    if (dt == 0.0) return M(0, 0, 0, 0);
    double r = 1.0 / dt;
    return M(A.d * r, -A.b * r, -A.c * r, A.a * r);
}
static inline m2 ldm(const double *a, int i) { return M(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]); }

/* ------------------------------------------------------------------ core/math.py */
/* ds_from_nodes, core/math.py:34-38 */
static inline m2 ds_from_nodes(v2 p0, v2 p1, v2 p2) {
    return M(p1.x - p0.x, p2.x - p0.x, p1.y - p0.y, p2.y - p0.y);
}
/* dF_from_dir, core/math.py:41-64 */
static inline m2 dF_from_dir(int n, int c, m2 B) {
    double a = 0.0, b = 0.0;
    if (n == 0) { a = -1.0; b = -1.0; }
    else if (n == 1) { a = 1.0; }
    else { b = 1.0; }
    m2 dDs = (c == 0) ? M(a, b, 0.0, 0.0) : M(0.0, 0.0, a, b);
    return mmul(dDs, B);
}
/* dF_from_vec6, core/math.py:67-72 */
static inline m2 dF_from_vec6(const double p[6], m2 B) {
    return mmul(M(p[2] - p[0], p[4] - p[0], p[3] - p[1], p[5] - p[1]), B);
}
/* nh_dPsidF, core/math.py:75-81 */
static inline m2 nh_dPsidF(m2 F, double mu, double la) {
    double J = det2(F);
    double logJ = log(fmax_(J, LOG_EPS));
    m2 FinvT = mT(inv2(F));
    return madd(msc(mu, F), msc(la * logJ - mu, FinvT));
}
/* nh_d2PsidF2_dir, core/math.py:84-93 */
static inline m2 nh_d2(m2 F, m2 dF, double mu, double la) {
    double J = det2(F);
    double logJ = log(fmax_(J, LOG_EPS));
    m2 Finv = inv2(F);
    m2 G = mT(Finv);
    double GdF = ddot(G, dF);
    m2 GdFtG = mmul(mmul(G, mT(dF)), G);
    return msub(madd(msc(mu, dF), msc(la * GdF, G)), msc(la * logJ - mu, GdFtG));
}
/* nh_pHp_elem, core/math.py:96-100 */
static inline double nh_pHp_elem(m2 F, m2 B, const double p[6], double mu, double la) {
    m2 dF = dF_from_vec6(p, B);
    return ddot(dF, nh_d2(F, dF, mu, la));
}
/* barrier_b / barrier_bp / barrier_bpp, core/math.py:112-129 */
static inline double barrier_b(double d, double dhat) { double u = d - dhat; return -(u * u) * log(d / dhat); }
static inline double barrier_bp(double d, double dhat) {
    double u = d - dhat; return -2.0 * u * log(d / dhat) - (u * u) / d;
}
static inline double barrier_bpp(double d, double dhat) {
    double u = d - dhat; return -2.0 * log(d / dhat) - 4.0 * u / d + (u * u) / (d * d);
}
/* pair_mu, core/math.py:132-144 */
static inline double pair_mu(double mu, int per_body, const double *mu_node, int i, int j) {
    if (per_body == 0) return mu;
    double mi = mu_node[i], mj = mu_node[j], sm = mi + mj;
    if (sm > 0.0) return 2.0 * mi * mj / sm;
    return 0.0;
}

/* ------------------------------------------------------------------ core/sdf.py */
typedef struct { double d; v2 g; m2 H; } sdfhit;

/* _seg_closest, core/sdf.py:22-34 */
static inline double seg_closest(v2 p, v2 a, v2 b, v2 *q, double *isv) {
    v2 ab = sub(b, a);
    double t = dot(sub(p, a), ab) / fmax_(dot(ab, ab), 1.0e-30);
    double tc = fmin_(fmax_(t, 0.0), 1.0);
    *q = add(a, scl(tc, ab));
    *isv = (t <= 0.0 || t >= 1.0) ? 1.0 : 0.0;
    return len(sub(p, *q));
}

/* sdf_eval, core/sdf.py:44-137 */
static sdfhit sdf_eval(int kind, double cx, double cy, double rx, double ry, double rref, v2 x) {
    sdfhit h;
    h.d = 0.0; h.g = V(0, 0); h.H = M(0, 0, 0, 0);
    if (kind == 0) {
        v2 diff = sub(x, V(cx, cy)); double dc = len(diff); v2 nh = vdiv(diff, dc);
        h.d = dc - rx; h.g = nh;
        m2 I_nn = msub(M(1.0, 0.0, 0.0, 1.0), M(nh.x * nh.x, nh.x * nh.y, nh.y * nh.x, nh.y * nh.y));
        double r = 1.0 / dc;
        h.H = M(I_nn.a * r, I_nn.b * r, I_nn.c * r, I_nn.d * r);
    } else if (kind == 1) {
        double ux = (x.x - cx) / rx, uy = (x.y - cy) / ry;
        double u = ux * ux + uy * uy, su = sqrt(fmax_(u, 1.0e-18));
        v2 w = V((x.x - cx) / (rx * rx), (x.y - cy) / (ry * ry));
        h.d = rref * (su - 1.0); h.g = scl(rref / su, w);
        m2 D = M(1.0 / (rx * rx), 0.0, 0.0, 1.0 / (ry * ry));
        double iu = 1.0 / u;
        m2 ww = M(w.x * w.x, w.x * w.y, w.y * w.x, w.y * w.y);
        h.H = msc(rref / su, msub(D, msc(iu, ww)));
    } else if (kind == 4) {
        v2 n = V(rx, ry);
        h.d = dot(n, sub(x, V(cx, cy))); h.g = n;
        h.H = M(0, 0, 0, 0);
    } else {
        double r = fmin_(fmax_(rref, 0.0), fmin_(rx, ry));
        double sx = 1.0; if (x.x < cx) sx = -1.0;
        double sy = 1.0; if (x.y < cy) sy = -1.0;
        double qx = sx * (x.x - cx) - (rx - r);
        double qy = sy * (x.y - cy) - (ry - r);
        double mx = fmax_(qx, 0.0), my = fmax_(qy, 0.0);
        double ml = sqrt(mx * mx + my * my);
        h.d = ml + fmin_(fmax_(qx, qy), 0.0) - r;
        if (ml > 1.0e-12) {
            double gx = mx / ml, gy = my / ml;
            h.g = V(sx * gx, sy * gy);
            if (qx > 0.0 && qy > 0.0) {
                double off = -gx * gy / ml;
                h.H = M(gy * gy / ml, sx * sy * off, sx * sy * off, gx * gx / ml);
            } else {
                h.H = M(0, 0, 0, 0);
            }
        } else {
            if (qx > qy) h.g = V(sx, 0.0); else h.g = V(0.0, sy);
            h.H = M(0, 0, 0, 0);
        }
    }
    if (kind == 3) {
        double r3 = fmin_(fmax_(rref, 0.0), rx * 0.5);
        double rin = rx - r3;
        v2 c0 = V(cx, cy);
        double a0 = 1.5707963267948966;
        v2 v0 = add(c0, scl(rin, V(cos(a0), sin(a0))));
        v2 v1 = add(c0, scl(rin, V(cos(a0 + 2.0943951023931953), sin(a0 + 2.0943951023931953))));
        v2 vv2 = add(c0, scl(rin, V(cos(a0 + 4.1887902047863905), sin(a0 + 4.1887902047863905))));
        v2 q0, q1, q2; double s0, s1, s2;
        double d0 = seg_closest(x, v0, v1, &q0, &s0);
        double d1 = seg_closest(x, v1, vv2, &q1, &s1);
        double d2 = seg_closest(x, vv2, v0, &q2, &s2);
        double dm = d0; v2 qm = q0; double sm = s0;
        if (d1 < dm) { dm = d1; qm = q1; sm = s1; }
        if (d2 < dm) { dm = d2; qm = q2; sm = s2; }
        v2 e0 = sub(v1, v0), e1 = sub(vv2, v1), e2 = sub(v0, vv2);
        v2 p0 = sub(x, v0), p1 = sub(x, v1), p2 = sub(x, vv2);
        double k0 = e0.x * p0.y - e0.y * p0.x;
        double k1 = e1.x * p1.y - e1.y * p1.x;
        double k2 = e2.x * p2.y - e2.y * p2.x;
        double sgn = 1.0;
        if (k0 >= 0.0 && k1 >= 0.0 && k2 >= 0.0) sgn = -1.0;
        double dl = fmax_(dm, 1.0e-30);
        h.d = sgn * dm - r3;
        h.g = scl(sgn / dl, sub(x, qm));
        if (sm > 0.5 && sgn > 0.0) {
            v2 gg = h.g;
            m2 I_gg = msub(M(1.0, 0.0, 0.0, 1.0), M(gg.x * gg.x, gg.x * gg.y, gg.y * gg.x, gg.y * gg.y));
            double r = 1.0 / dl;
            h.H = M(I_gg.a * r, I_gg.b * r, I_gg.c * r, I_gg.d * r);
        } else {
            h.H = M(0, 0, 0, 0);
        }
    }
    return h;
}

typedef struct { int kind; double cx, cy, rx, ry, rref, r, mu; } collider;
static inline collider col_at(const d2o_solver *s, int k) {
    const double *c = s->colliders + 8 * k;
    collider o = {(int)c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7]};
    return o;
}

/* ------------------------------------------------------------------ step setup, kernels.py:41-68 */
static void init_step(d2o_solver *s) {
    double ddr = s->dt * s->drag;
    for (int i = 0; i < s->N; ++i) {
        v2 xi = ld(s->x, i);
        st(s->xn, i, xi);
        st(s->xhat, i, add(xi, scl(ddr, ld(s->v, i))));
    }
}
static void apply_bc(d2o_solver *s) {
    for (int b = 0; b < s->n_bc; ++b) {
        int n = s->bc_idx[b];
        v2 t = ld(s->bc_target, b);
        st(s->x, n, t); st(s->xhat, n, t);
    }
}

/* ------------------------------------------------------------------ gradient + diagonal */
/* grad_diag_mass_kernel, kernels.py:72-82 */
static void grad_diag_mass(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i) {
        st(s->grad_prev, i, ld(s->grad, i));
        double m = s->mass[i];
        v2 d = sub(ld(s->x, i), ld(s->xhat, i));
        st(s->grad, i, cw(V(m * d.x, m * d.y), ld(s->free_, i)));
        st(s->diagH, i, V(m, m));
    }
}
/* grad_diag_elastic_kernel, kernels.py:85-128 (clamp = 1) */
static void grad_diag_elastic(d2o_solver *s) {
    const double h2 = s->h2;
    for (int t = 0; t < s->T; ++t) {
        int i0 = s->tri[3 * t], i1 = s->tri[3 * t + 1], i2 = s->tri[3 * t + 2];
        v2 p0 = ld(s->x, i0), p1 = ld(s->x, i1), p2 = ld(s->x, i2);
        m2 Bt = ldm(s->Bm, t);
        m2 F = mmul(ds_from_nodes(p0, p1, p2), Bt);
        double A = s->area[t], m_ = s->mu[t], l_ = s->lam[t];
        m2 P = nh_dPsidF(F, m_, l_);
        m2 HH = msc(A, mmul(P, mT(Bt)));
        v2 g1 = V(HH.a, HH.c), g2 = V(HH.b, HH.d);
        v2 g0 = V(-(g1.x + g2.x), -(g1.y + g2.y));
        atomic_add2(s->grad, i0, scl(h2, g0));
        atomic_add2(s->grad, i1, scl(h2, g1));
        atomic_add2(s->grad, i2, scl(h2, g2));
        int ids[3] = {i0, i1, i2};
        for (int n = 0; n < 3; ++n) {
            m2 dFx = dF_from_dir(n, 0, Bt);
            double dx = A * ddot(dFx, nh_d2(F, dFx, m_, l_));
            m2 dFy = dF_from_dir(n, 1, Bt);
            double dy = A * ddot(dFy, nh_d2(F, dFy, m_, l_));
            dx = fmax_(dx, 0.0); dy = fmax_(dy, 0.0);
            atomic_add2(s->diagH, ids[n], V(h2 * dx, h2 * dy));
        }
    }
}
/* grad_diag_disc_kernel, kernels.py:131-157 */
static void grad_diag_disc(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        v2 diff = sub(ld(s->x, n), V(c.cx, c.cy));
        double dc = len(diff), d = dc - c.r;
        if (d <= 0.0 || d >= s->dhat) continue;
        v2 nh = vdiv(diff, dc);
        double bp = barrier_bp(d, s->dhat), bpp = barrier_bpp(d, s->dhat);
        atomic_add2(s->grad, n, scl(s->h2 * s->kappa * bp, nh));
        double tang = bp / dc;
        double dgx = s->kappa * (bpp * nh.x * nh.x + tang * (1.0 - nh.x * nh.x));
        double dgy = s->kappa * (bpp * nh.y * nh.y + tang * (1.0 - nh.y * nh.y));
        dgx = fmax_(dgx, 0.0); dgy = fmax_(dgy, 0.0);
        atomic_add2(s->diagH, n, V(s->h2 * dgx, s->h2 * dgy));
    }
}
/* grad_diag_sdf_kernel, core/sdf.py:140-154 */
static void grad_diag_sdf(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        sdfhit h = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, ld(s->x, n));
        if (h.d <= 0.0 || h.d >= s->dhat) continue;
        double bp = barrier_bp(h.d, s->dhat), bpp = barrier_bpp(h.d, s->dhat);
        atomic_add2(s->grad, n, scl(s->h2 * s->kappa * bp, h.g));
        double dgx = s->kappa * (bpp * h.g.x * h.g.x + bp * h.H.a);
        double dgy = s->kappa * (bpp * h.g.y * h.g.y + bp * h.H.d);
        dgx = fmax_(dgx, 0.0); dgy = fmax_(dgy, 0.0);
        atomic_add2(s->diagH, n, V(s->h2 * dgx, s->h2 * dgy));
    }
}
/* grad_friction_disc_kernel, kernels.py:640-681 */
static void grad_friction_disc(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        v2 fr = ld(s->free_, n);
        if (fr.x <= 0.5 && fr.y <= 0.5) continue;
        v2 diff = sub(ld(s->x, n), V(c.cx, c.cy));
        double dc = len(diff), d = dc - c.r;
        if (d <= 0.0 || d >= s->dhat) continue;
        v2 nh = vdiv(diff, dc);
        double f_n = s->kappa * fabs_(barrier_bp(d, s->dhat));
        v2 v = vsc(sub(ld(s->x, n), ld(s->xn, n)), s->inv_dt);
        double vn = dot(v, nh);
        v2 vt = sub(v, scl(vn, nh));
        double vtmag = len(vt);
        v2 tdir = vdiv(vt, fmax_(vtmag, s->epsv));
        atomic_add2(s->grad, n, cw(scl(s->h2 * c.mu * f_n, tdir), fr));
        double kt = s->h2 * c.mu * f_n * s->inv_dt / fmax_(vtmag, s->epsv);
        v2 th = V(-nh.y, nh.x);
        atomic_add2(s->diagH, n, cw(V(kt * th.x * th.x, kt * th.y * th.y), fr));
    }
}
/* _sdf_fric_frame, core/sdf.py:200-210 */
static inline void sdf_fric_frame(sdfhit h, v2 xk, v2 xkm1, double kappa, double dhat, double inv_dt,
                                  double *f_n, v2 *nh, v2 *vt, double *vtm) {
    double gn = len(h.g);
    *nh = vdiv(h.g, fmax_(gn, 1.0e-30));
    *f_n = kappa * fabs_(barrier_bp(h.d, dhat)) * gn;
    v2 vel = vsc(sub(xk, xkm1), inv_dt);
    *vt = sub(vel, scl(dot(vel, *nh), *nh));
    *vtm = len(*vt);
}
/* grad_friction_sdf_kernel, core/sdf.py:213-233 */
static void grad_friction_sdf(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        v2 fr = ld(s->free_, n);
        if (fr.x <= 0.5 && fr.y <= 0.5) continue;
        sdfhit h = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, ld(s->x, n));
        if (h.d <= 0.0 || h.d >= s->dhat) continue;
        double f_n, vtm; v2 nh, vt;
        sdf_fric_frame(h, ld(s->x, n), ld(s->xn, n), s->kappa, s->dhat, s->inv_dt, &f_n, &nh, &vt, &vtm);
        v2 tdir = vdiv(vt, fmax_(vtm, s->epsv));
        atomic_add2(s->grad, n, cw(scl(s->h2 * c.mu * f_n, tdir), fr));
        double kt = s->h2 * c.mu * f_n * s->inv_dt / fmax_(vtm, s->epsv);
        v2 th = V(-nh.y, nh.x);
        atomic_add2(s->diagH, n, cw(V(kt * th.x * th.x, kt * th.y * th.y), fr));
    }
}

/* ------------------------------------------------------------------ ExternalForce, actuation.py:37-50 */
static void ext_grad(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i)
        st(s->grad, i, sub(ld(s->grad, i), scl(s->h2, ld(s->fext, i))));
}
static void ext_energy(d2o_solver *s, double *E) {
    for (int i = 0; i < s->N; ++i)
        E[s->node2env[i]] += -s->h2 * dot(ld(s->fext, i), sub(ld(s->x, i), ld(s->xn, i)));
}

/* ------------------------------------------------------------------ IPC, implicit/ipc_contact.py */
/* _seg_dist, ipc_contact.py:94-99 */
static inline double seg_dist(v2 p, v2 a, v2 b) {
    v2 ab = sub(b, a);
    double t = dot(sub(p, a), ab) / fmax_(dot(ab, ab), 1.0e-30);
    t = fmin_(fmax_(t, 0.0), 1.0);
    return len(sub(sub(p, a), scl(t, ab)));
}
/* _accd, ipc_contact.py:102-127 */
static double accd(v2 p, v2 a, v2 b, v2 dp, v2 da, v2 db, double g, double t_c) {
    v2 m = vdiv(add(add(dp, da), db), 3.0);
    dp = sub(dp, m); da = sub(da, m); db = sub(db, m);
    double lp = len(dp) + fmax_(len(da), len(db));
    if (lp <= 1.0e-30) return t_c;
    double d = seg_dist(p, a, b);
    double t = 0.0, tl = (d - g) / lp;
    for (int k = 0; k < 32; ++k) {
        double tn = t + tl;
        if (tn >= t_c) return t_c;
        d = seg_dist(add(p, scl(tn, dp)), add(a, scl(tn, da)), add(b, scl(tn, db)));
        if (k > 0 && d < g) return t;
        t = tn;
        tl = 0.9 * d / lp;
    }
    return t;
}

typedef struct {
    d2o_solver *s;
    int mode;
    const double *pdir;
    double *E, *clr, *alpha;
    double *grad, *diagH;
    const double *free_;
    double mu, h2, floor_, tc0;
    int per_body;
} ipc_launch;

/* _pair, ipc_contact.py:130-171 */
static void ipc_pair_term(const ipc_launch *L, double coef, int ip, int ia, int ib, double wa, double wb,
                          double d, v2 n, double ddd, int e, double mu) {
    d2o_solver *s = L->s;
    const double dhat = s->ipc_dhat, kappa = s->ipc_kappa, inv_dt = s->inv_dt, epsv = s->epsv, h2 = L->h2;
    double bp = barrier_bp(d, dhat);
    double f_n = -kappa * bp;
    v2 tn = V(-n.y, n.x);
    v2 u = sub(sub(sub(ld(s->x, ip), ld(s->xn, ip)), scl(wa, sub(ld(s->x, ia), ld(s->xn, ia)))),
               scl(wb, sub(ld(s->x, ib), ld(s->xn, ib))));
    double ut = dot(u, tn);
    double vt = fabs_(ut) * inv_dt;
    double kt = mu * f_n * inv_dt / fmax_(vt, epsv);
    if (L->mode == 0) {
        double bpp = barrier_bpp(d, dhat);
        v2 g = scl(h2, add(scl(-f_n, n), scl(mu * f_n * (ut * inv_dt / fmax_(vt, epsv)), tn)));
        v2 hd = scl(h2, V(kappa * bpp * n.x * n.x + kt * tn.x * tn.x, kappa * bpp * n.y * n.y + kt * tn.y * tn.y));
        atomic_add2(L->grad, ip, scl(coef, cw(g, ld(L->free_, ip))));
        atomic_add2(L->diagH, ip, scl(coef, hd));
        atomic_add2(L->grad, ia, scl(-coef * wa, cw(g, ld(L->free_, ia))));
        atomic_add2(L->diagH, ia, scl(coef * wa * wa, hd));
        atomic_add2(L->grad, ib, scl(-coef * wb, cw(g, ld(L->free_, ib))));
        atomic_add2(L->diagH, ib, scl(coef * wb * wb, hd));
    } else if (L->mode == 1) {
        double bpp = barrier_bpp(d, dhat);
        v2 dq = sub(sub(ld(L->pdir, ip), scl(wa, ld(L->pdir, ia))), scl(wb, ld(L->pdir, ib)));
        double dn = dot(dq, n), dt_ = dot(dq, tn);
        double val = fmax_(kappa * (bpp * dn * dn + bp * ddd), 0.0);
        s->pHp[e] = s->pHp[e] + coef * h2 * (val + kt * dt_ * dt_);
    } else {
        double asl = epsv / inv_dt;
        double au = fabs_(ut);
        double f0 = au - 0.5 * asl;
        if (au < asl) f0 = au * au / (2.0 * asl);
        L->E[e] = L->E[e] + coef * h2 * (kappa * barrier_b(d, dhat) + mu * f_n * f0);
    }
}

static int excluded(const d2o_solver *s, int slot, int local) {
    /* is boundary-local `local` in slot's sorted exclusion list? */
    int lo = s->excl_ptr[slot], hi = s->excl_ptr[slot + 1];
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        int v = s->excl_idx[mid];
        if (v == local) return 1;
        if (v < local) lo = mid + 1; else hi = mid;
    }
    return 0;
}

/* ipc_pair_kernel, ipc_contact.py:174-296. Candidates are the boundary nodes of the edge's
 * environment in ascending slot order (a superset of the hash-grid query: every candidate
 * is filtered by its exact distance below). */
static void ipc_pair(const ipc_launch *L) {
    d2o_solver *s = L->s;
    const int mode = L->mode;
    const double dhat = s->ipc_dhat, reach = s->reach, gap = s->gap;
    for (int k = 0; k < s->Ne; ++k) {
        int a = s->ea[k], b = s->eb[k], e = s->e2env[k];
        int start = s->bstart[e], n_be = s->bpe[e];
        v2 xa = ld(s->x, a), xb = ld(s->x, b);
        v2 ab = sub(xb, xa);
        double L2 = fmax_(dot(ab, ab), 1.0e-30);
        double Ll = sqrt(L2);
        double dlo = 1.0e-9 * dhat;
        double onset = 0.02 * dhat;
        double t_c = g_tc_fixed ? L->tc0 : L->alpha[e];
        for (int jl = 0; jl < n_be; ++jl) {
            int jb = start + jl;
            int pn = s->bnd[jb];
            int ok = (s->b2e[jb] == e) && pn != a && pn != b;
            if (ok) ok = !excluded(s, jb, s->ela[k]) && !excluded(s, jb, s->elb[k]);
            if (!ok) continue;
            v2 xp = ld(s->x, pn);
            v2 w = sub(xp, xa);
            double tt = dot(w, ab) / L2;
            v2 dvec = sub(w, scl(tt, ab));
            if (tt <= 0.0) dvec = w;
            else if (tt >= 1.0) dvec = sub(xp, xb);
            double d = len(dvec);
            if (!(d < reach)) continue;
            if (mode == 1 || mode == 3) {
                amin(L->clr, e, d);
                double keep = fmax_(gap * d, dhat - onset);
                if (d < dhat) keep = d - fmin_(2.0 * (dhat - d) + onset, 0.5 * d);
                if (mode == 3) keep = fmin_(d, fmax_(gap * d, L->floor_));
                amin(L->alpha, e, accd(xp, xa, xb, ld(L->pdir, pn), ld(L->pdir, a), ld(L->pdir, b), keep, t_c));
            }
            if (mode != 3) {
                double mu_p = pair_mu(L->mu, L->per_body, s->mu_node, pn, a);
                if (tt > 0.0 && tt < 1.0 && d < dhat) {
                    d = fmax_(d, dlo);
                    double ddd = 0.0;
                    if (mode == 1) {
                        v2 de = sub(ld(L->pdir, b), ld(L->pdir, a));
                        v2 dw = sub(ld(L->pdir, pn), ld(L->pdir, a));
                        double c0 = cross2(ab, w);
                        double c1 = cross2(de, w) + cross2(ab, dw);
                        double c2 = 2.0 * cross2(de, dw);
                        double L1 = dot(ab, de) / Ll;
                        double Lq = (dot(de, de) - L1 * L1) / Ll;
                        double s0 = c0 / Ll;
                        double s1 = (c1 - s0 * L1) / Ll;
                        ddd = (c2 - 2.0 * s1 * L1 - s0 * Lq) / Ll;
                        if (c0 < 0.0) ddd = -ddd;
                    }
                    ipc_pair_term(L, 1.0, pn, a, b, 1.0 - tt, tt, d, vdiv(dvec, d), ddd, e, mu_p);
                }
                double coef_a = -s->ca[k];
                if (tt <= 0.0) coef_a = coef_a + 1.0;
                double d_a = len(w);
                if (coef_a != 0.0 && d_a < dhat) {
                    d_a = fmax_(d_a, dlo);
                    v2 n_a = vdiv(w, d_a);
                    double ddd = 0.0;
                    if (mode == 1) {
                        v2 dw = sub(ld(L->pdir, pn), ld(L->pdir, a));
                        double dn = dot(dw, n_a);
                        ddd = (dot(dw, dw) - dn * dn) / d_a;
                    }
                    ipc_pair_term(L, coef_a, pn, a, b, 1.0, 0.0, d_a, n_a, ddd, e, mu_p);
                }
                double coef_b = -s->cb[k];
                if (tt >= 1.0) coef_b = coef_b + 1.0;
                v2 wb_ = sub(xp, xb);
                double d_b = len(wb_);
                if (coef_b != 0.0 && d_b < dhat) {
                    d_b = fmax_(d_b, dlo);
                    v2 n_b = vdiv(wb_, d_b);
                    double ddd = 0.0;
                    if (mode == 1) {
                        v2 dw = sub(ld(L->pdir, pn), ld(L->pdir, b));
                        double dn = dot(dw, n_b);
                        ddd = (dot(dw, dw) - dn * dn) / d_b;
                    }
                    ipc_pair_term(L, coef_b, pn, a, b, 0.0, 1.0, d_b, n_b, ddd, e, mu_p);
                }
            }
        }
    }
}
/* ipc_far_cap_kernel, ipc_contact.py:299-305 */
static void ipc_far_cap(d2o_solver *s, const double *p_inf, double *alpha) {
    for (int e = 0; e < s->B; ++e)
        if (p_inf[e] > 0.0) alpha[e] = fmin_(alpha[e], 0.45 * s->reach / p_inf[e]);
}
static ipc_launch ipc_base(d2o_solver *s, int mode, const double *pdir, double *E, double *clr, double *alpha) {
    ipc_launch L;
    L.s = s; L.mode = mode; L.pdir = pdir; L.E = E; L.clr = clr; L.alpha = alpha;
    L.grad = s->grad; L.diagH = s->diagH; L.free_ = s->free_;
    L.mu = s->friction ? s->ipc_mu : 0.0;
    L.per_body = s->friction ? s->per_body : 0;
    L.h2 = s->h2;
    L.floor_ = (mode == 3) ? s->bc_floor * s->ipc_dhat : 0.0;
    L.tc0 = (mode == 3) ? 1.0 : s->alpha_max;
    return L;
}
/* IPCContact.ccd, ipc_contact.py:432-439 */
static void ipc_ccd(d2o_solver *s, const double *pdir, const double *p_inf, double *alpha) {
    for (int e = 0; e < s->B; ++e) { alpha[e] = 1.0; s->clr[e] = 1.0e30; }
    ipc_launch L = ipc_base(s, 3, pdir, s->Ener, s->clr, alpha);
    ipc_pair(&L);
    ipc_far_cap(s, p_inf, alpha);
}
/* IPCContact._sweep + bc_motion/bc_advance, ipc_contact.py:308-331, 456-463 */
static void ipc_sweep(d2o_solver *s) {
    for (int e = 0; e < s->B; ++e) s->q_inf[e] = 0.0;
    for (int b = 0; b < s->n_bc; ++b) {
        int i = s->bc_idx[b];
        v2 d = sub(ld(s->bc_target, b), ld(s->x, i));
        st(s->q, i, d);
        amax(s->q_inf, s->node2env[i], len(d));
    }
    ipc_ccd(s, s->q, s->q_inf, s->sweep_beta);
    for (int b = 0; b < s->n_bc; ++b) {
        int i = s->bc_idx[b];
        double t = s->sweep_beta[s->node2env[i]];
        if (t >= 1.0) st(s->x, i, ld(s->bc_target, b));
        else st(s->x, i, add(ld(s->x, i), scl(t, sub(ld(s->bc_target, b), ld(s->x, i)))));
        st(s->xhat, i, ld(s->x, i));
    }
}
static int all_beta_done(const d2o_solver *s) {
    for (int e = 0; e < s->B; ++e) if (!(s->sweep_beta[e] >= 1.0)) return 0;
    return 1;
}

/* ------------------------------------------------------------------ Tendon, actuation.py:169-316 */
static inline void seg_dir(v2 xa, v2 xb, double out[3]) {
    v2 t = sub(xb, xa);
    double ln = fmax_(len(t), 1.0e-12);
    out[0] = t.x / ln; out[1] = t.y / ln; out[2] = 1.0 / ln;
}
static void tendon_lengths(d2o_solver *s) {
    for (int k = 0; k < s->n_tendon; ++k) s->t_L[k] = 0.0;
    for (int j = 0; j < s->n_tent; ++j) {
        int k = s->t_nxt[j];
        if (k >= 0) s->t_L[s->t_tid[j]] += len(sub(ld(s->x, s->t_node[k]), ld(s->x, s->t_node[j])));
    }
}
static void tendon_grad(d2o_solver *s) {
    tendon_lengths(s);
    for (int k = 0; k < s->n_tendon; ++k) {
        if (s->t_stiff[k] > 0.0) {
            double ext = s->t_L[k] - s->t_L0[k];
            if (ext > 0.0) { s->t_tau[k] = s->t_stiff[k] * ext; s->t_keff[k] = s->t_stiff[k]; }
            else { s->t_tau[k] = 0.0; s->t_keff[k] = 0.0; }
        } else {
            s->t_tau[k] = fmax_(s->t_Tcmd[k], 0.0); s->t_keff[k] = 0.0;
        }
    }
    for (int j = 0; j < s->n_tent; ++j) {
        int n = s->t_node[j], k = s->t_tid[j];
        v2 gL = V(0, 0), geo = V(0, 0);
        if (s->t_prv[j] >= 0) {
            double sp[3]; seg_dir(ld(s->x, s->t_node[s->t_prv[j]]), ld(s->x, n), sp);
            gL = add(gL, V(sp[0], sp[1]));
            geo = add(geo, V((1.0 - sp[0] * sp[0]) * sp[2], (1.0 - sp[1] * sp[1]) * sp[2]));
        }
        if (s->t_nxt[j] >= 0) {
            double sn[3]; seg_dir(ld(s->x, n), ld(s->x, s->t_node[s->t_nxt[j]]), sn);
            gL = sub(gL, V(sn[0], sn[1]));
            geo = add(geo, V((1.0 - sn[0] * sn[0]) * sn[2], (1.0 - sn[1] * sn[1]) * sn[2]));
        }
        atomic_add2(s->grad, n, scl(s->h2 * s->t_tau[k], gL));
        atomic_add2(s->diagH, n, V(s->h2 * (s->t_tau[k] * geo.x + s->t_keff[k] * gL.x * gL.x),
                                   s->h2 * (s->t_tau[k] * geo.y + s->t_keff[k] * gL.y * gL.y)));
    }
}
static void tendon_pHp(d2o_solver *s) {
    for (int k = 0; k < s->n_tendon; ++k) s->t_dL[k] = 0.0;
    for (int j = 0; j < s->n_tent; ++j) {
        int m = s->t_nxt[j];
        if (m < 0) continue;
        int k = s->t_tid[j];
        double sd[3]; seg_dir(ld(s->x, s->t_node[j]), ld(s->x, s->t_node[m]), sd);
        v2 d = V(sd[0], sd[1]);
        v2 dp = sub(ld(s->p, s->t_node[m]), ld(s->p, s->t_node[j]));
        double along = dot(dp, d);
        s->t_dL[k] += along;
        s->pHp[s->t2env[k]] += s->h2 * s->t_tau[k] * (dot(dp, dp) - along * along) * sd[2];
    }
    for (int k = 0; k < s->n_tendon; ++k)
        s->pHp[s->t2env[k]] += s->h2 * s->t_keff[k] * s->t_dL[k] * s->t_dL[k];
}
static void tendon_energy(d2o_solver *s, double *E) {
    tendon_lengths(s);
    for (int k = 0; k < s->n_tendon; ++k) {
        if (s->t_stiff[k] > 0.0) {
            double ext = s->t_L[k] - s->t_L0[k];
            if (ext > 0.0) E[s->t2env[k]] += 0.5 * s->h2 * s->t_stiff[k] * ext * ext;
        } else {
            E[s->t2env[k]] += s->h2 * fmax_(s->t_Tcmd[k], 0.0) * s->t_L[k];
        }
    }
}

/* ------------------------------------------------------------------ AffineBodies, affine.py */
typedef struct { double m[6][6]; } m6;
/* reduced_hessian, affine.py:60-101 */
static m6 reduced_hessian(m2 A, double Mu, double La, double h2, const double *Hx, const double *Hy) {
    m6 H; memset(&H, 0, sizeof H);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) { H.m[r][c] = Hx[3 * r + c]; H.m[r + 3][c + 3] = Hy[3 * r + c]; }
    const int idx[4] = {1, 2, 4, 5};
    for (int k = 0; k < 4; ++k) {
        m2 E = M(k == 0, k == 1, k == 2, k == 3);
        m2 col = nh_d2(A, E, Mu, La);
        double cv[4] = {col.a, col.b, col.c, col.d};
        for (int r = 0; r < 4; ++r) H.m[idx[r]][idx[k]] = H.m[idx[r]][idx[k]] + h2 * cv[r];
    }
    double a = A.a + A.d, b = A.c - A.b;
    double n = sqrt(a * a + b * b);
    if (n > 1.0e-12) {
        double f = 0.7071067811865476 / n;
        double t[4] = {-b * f, -a * f, a * f, -b * f};
        m2 Tm = M(t[0], t[1], t[2], t[3]);
        double lam_t = ddot(Tm, nh_d2(A, Tm, Mu, La));
        if (lam_t < 0.0)
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c)
                    H.m[idx[r]][idx[c]] = H.m[idx[r]][idx[c]] - h2 * lam_t * t[r] * t[c];
    }
    return H;
}
/* chol6, affine.py:104-129 */
static m6 chol6(const m6 *H) {
    m6 L; memset(&L, 0, sizeof L);
    int ok = 1;
    for (int j = 0; j < 6; ++j) {
        double s = H->m[j][j];
        for (int k = 0; k < j; ++k) s = s - L.m[j][k] * L.m[j][k];
        if (s <= 1.0e-9 * fabs_(H->m[j][j]) || s <= 0.0) ok = 0;
        if (ok) {
            double d = sqrt(s);
            L.m[j][j] = d;
            for (int i = j + 1; i < 6; ++i) {
                double v = H->m[i][j];
                for (int k = 0; k < j; ++k) v = v - L.m[i][k] * L.m[j][k];
                L.m[i][j] = v / d;
            }
        }
    }
    if (!ok) {
        memset(&L, 0, sizeof L);
        for (int j = 0; j < 6; ++j) L.m[j][j] = sqrt(fmax_(H->m[j][j], 1.0e-30));
    }
    return L;
}
/* chol6_solve, affine.py:132-147 */
static void chol6_solve(const m6 *L, const double b[6], double x[6]) {
    double y[6];
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s = s - L->m[i][k] * y[k];
        y[i] = s / L->m[i][i];
    }
    for (int ii = 0; ii < 6; ++ii) {
        int i = 5 - ii;
        double s = y[i];
        for (int k = i + 1; k < 6; ++k) s = s - L->m[k][i] * x[k];
        x[i] = s / L->m[i][i];
    }
}
/* The 6x6 block algebra alone, for tests/test_rigid.py:62-94's checks: H (36, row-major) =
   reduced_hessian(A (a11 a12 a21 a22), Mu, La, h2, Hx, Hy (9 each)); x = chol6_solve(chol6(H), b). */
void d2o_affine_hessian(const double *A4, double Mu, double La, double h2, const double *Hx, const double *Hy,
                        double *H36) {
    m6 H = reduced_hessian(M(A4[0], A4[1], A4[2], A4[3]), Mu, La, h2, Hx, Hy);
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) H36[6 * r + c] = H.m[r][c];
}
void d2o_chol6_solve(const double *H36, const double *b, double *x) {
    m6 H;
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) H.m[r][c] = H36[6 * r + c];
    m6 L = chol6(&H);
    chol6_solve(&L, b, x);
}
static inline double dot6(const double *a, const double *b) {
    double s = a[0] * b[0];
    for (int k = 1; k < 6; ++k) s = s + a[k] * b[k];
    return s;
}
static inline m2 A_of(const double *q) { return M(q[1], q[2], q[4], q[5]); }

/* affine_expand_kernel, affine.py:215-224 */
static void affine_expand(d2o_solver *s, const double *v6all, double *out) {
    for (int k = 0; k < s->n_affn; ++k) {
        const double *w = s->a_w + 3 * k;
        const double *v = v6all + 6 * s->a_grp[k];
        st(out, s->a_node[k], V(w[0] * v[0] + w[1] * v[1] + w[2] * v[2], w[0] * v[3] + w[1] * v[4] + w[2] * v[5]));
    }
}
/* AffineBodies.gather + affine_gather_kernel, affine.py:156-175, 360-365 */
static void affine_gather(d2o_solver *s) {
    memcpy(s->a_gq_prev, s->a_gq, sizeof(double) * 6 * s->n_aff);
    memset(s->a_gq, 0, sizeof(double) * 6 * s->n_aff);
    memset(s->a_Hx, 0, sizeof(double) * 9 * s->n_aff);
    memset(s->a_Hy, 0, sizeof(double) * 9 * s->n_aff);
    for (int k = 0; k < s->n_affn; ++k) {
        int i = s->a_node[k], b = s->a_grp[k];
        const double *ww = s->a_w + 3 * k;
        v2 g = ld(s->grad, i), d = ld(s->diagH, i);
        double *gq = s->a_gq + 6 * b;
        double add6[6] = {g.x * ww[0], g.x * ww[1], g.x * ww[2], g.y * ww[0], g.y * ww[1], g.y * ww[2]};
        for (int r = 0; r < 6; ++r) gq[r] = gq[r] + add6[r];
        double *Hx = s->a_Hx + 9 * b, *Hy = s->a_Hy + 9 * b;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double o = ww[r] * ww[c];
                Hx[3 * r + c] = Hx[3 * r + c] + d.x * o;
                Hy[3 * r + c] = Hy[3 * r + c] + d.y * o;
            }
        st(s->grad, i, V(0.0, 0.0));
    }
}
/* affine_reduce_kernel, affine.py:178-205 */
static void affine_reduce(d2o_solver *s) {
    for (int b = 0; b < s->n_aff; ++b) {
        int e = s->a_env[b];
        double *q = s->a_q + 6 * b;
        m2 A = A_of(q);
        m2 P = nh_dPsidF(A, s->a_Mu[b], s->a_La[b]);
        double g[6], y[6], z[6], zy[6];
        double *gq = s->a_gq + 6 * b, *gqp = s->a_gq_prev + 6 * b, *pp = s->a_pq + 6 * b;
        double hp[6] = {s->h2 * 0.0, s->h2 * P.a, s->h2 * P.b, s->h2 * 0.0, s->h2 * P.c, s->h2 * P.d};
        for (int r = 0; r < 6; ++r) g[r] = gq[r] + hp[r];
        m6 H = reduced_hessian(A, s->a_Mu[b], s->a_La[b], s->h2, s->a_Hx + 9 * b, s->a_Hy + 9 * b);
        m6 L = chol6(&H);
        for (int r = 0; r < 6; ++r) y[r] = g[r] - gqp[r];
        chol6_solve(&L, g, z);
        chol6_solve(&L, y, zy);
        s->gPg[e] += dot6(g, z);
        s->g_p[e] += dot6(g, pp);
        s->g_Py[e] += dot6(g, zy);
        s->y_p[e] += dot6(y, pp);
        s->y_Py[e] += dot6(y, zy);
        memcpy(gq, g, sizeof g);
        memcpy(s->a_zq + 6 * b, z, sizeof z);
    }
}
/* affine_direction_kernel + expand, affine.py:208-212, 373-376 */
static void affine_direction(d2o_solver *s) {
    for (int b = 0; b < s->n_aff; ++b) {
        double bb = s->beta[s->a_env[b]];
        double *pq = s->a_pq + 6 * b, *zq = s->a_zq + 6 * b;
        for (int r = 0; r < 6; ++r) pq[r] = -zq[r] + bb * pq[r];
    }
    affine_expand(s, s->a_pq, s->p);
}
/* affine_pHp_kernel, affine.py:227-234 */
static void affine_pHp(d2o_solver *s) {
    for (int b = 0; b < s->n_aff; ++b) {
        m2 dA = A_of(s->a_pq + 6 * b);
        double val = ddot(dA, nh_d2(A_of(s->a_q + 6 * b), dA, s->a_Mu[b], s->a_La[b]));
        s->pHp[s->a_env[b]] += s->h2 * fmax_(val, 0.0);
    }
}
/* affine_energy_kernel, affine.py:237-246 */
static void affine_energy(d2o_solver *s, double *E) {
    for (int b = 0; b < s->n_aff; ++b) {
        m2 A = A_of(s->a_q + 6 * b);
        double Mu = s->a_Mu[b], La = s->a_La[b];
        double logJ = log(fmax_(det2(A), LOG_EPS));
        double psi = 0.5 * Mu * (ddot(A, A) - 2.0) - Mu * logJ + 0.5 * La * logJ * logJ;
        E[s->a_env[b]] += s->h2 * psi;
    }
}
/* affine_advance_kernel + expand, affine.py:249-257, 378-381 */
static void affine_advance(d2o_solver *s) {
    for (int b = 0; b < s->n_aff; ++b) {
        int e = s->a_env[b];
        if (s->active[e] == 0) continue;
        double *q = s->a_q + 6 * b, *pq = s->a_pq + 6 * b;
        double al = s->alpha[e];
        for (int r = 0; r < 6; ++r) q[r] = q[r] + al * pq[r];
    }
    affine_expand(s, s->a_q, s->x);
}
/* affine_trial_kernel + expand, affine.py:260-269, 386-389 */
static void affine_trial(d2o_solver *s) {
    for (int b = 0; b < s->n_aff; ++b) {
        int e = s->a_env[b];
        if (s->active[e] == 0) continue;
        double *q = s->a_q + 6 * b, *q0 = s->a_q0 + 6 * b, *pq = s->a_pq + 6 * b;
        double al = s->alpha[e];
        for (int r = 0; r < 6; ++r) q[r] = q0[r] + al * pq[r];
    }
    affine_expand(s, s->a_q, s->x);
}

/* ------------------------------------------------------------------ RigidModes, affine.py:404-563 */
static inline v2 arm(v2 x, const double *a) { return sub(x, V(a[0] / a[2], a[1] / a[2])); }
/* centroid_kernel + rigid_gather_kernel, affine.py:404-453 */
static void rigid_gather(d2o_solver *s) {
    memset(s->r_acc, 0, sizeof(double) * 3 * s->n_rig);
    memset(s->r_gq, 0, sizeof(double) * 3 * s->n_rig);
    memset(s->r_gq_prev, 0, sizeof(double) * 3 * s->n_rig);
    memset(s->r_Hc, 0, sizeof(double) * 9 * s->n_rig);
    for (int k = 0; k < s->n_rign; ++k) {
        int i = s->r_node[k];
        double m = s->mass[i];
        v2 xi = ld(s->x, i);
        double *a = s->r_acc + 3 * s->r_grp[k];
        a[0] = a[0] + m * xi.x; a[1] = a[1] + m * xi.y; a[2] = a[2] + m;
    }
    for (int k = 0; k < s->n_rign; ++k) {
        int i = s->r_node[k], b = s->r_grp[k];
        v2 rr = arm(ld(s->x, i), s->r_acc + 3 * b);
        v2 g = ld(s->grad, i), gp = ld(s->grad_prev, i);
        double m = s->mass[i];
        v2 d = sub(ld(s->diagH, i), ld(s->diag_el, i));
        double dx = fmax_(d.x, 0.0) + m;
        double dy = fmax_(d.y, 0.0) + m;
        double *gq = s->r_gq + 3 * b, *gqp = s->r_gq_prev + 3 * b, *H = s->r_Hc + 9 * b;
        gq[0] = gq[0] + g.x; gq[1] = gq[1] + g.y; gq[2] = gq[2] + (rr.x * g.y - rr.y * g.x);
        gqp[0] = gqp[0] + gp.x; gqp[1] = gqp[1] + gp.y; gqp[2] = gqp[2] + (rr.x * gp.y - rr.y * gp.x);
        double h[9] = {dx, 0.0, -dx * rr.y, 0.0, dy, dy * rr.x, -dx * rr.y, dy * rr.x,
                       dx * rr.y * rr.y + dy * rr.x * rr.x};
        for (int r = 0; r < 9; ++r) H[r] = H[r] + h[r];
    }
}
static inline double det3(const double *a) {
    return a[0] * (a[4] * a[8] - a[7] * a[5]) - a[1] * (a[3] * a[8] - a[6] * a[5]) + a[2] * (a[3] * a[7] - a[6] * a[4]);
}
static void inv3(const double *a, double *o) {
    double dt = det3(a);
    if (dt == 0.0) { memset(o, 0, 9 * sizeof(double)); return; }
    double b[9];
    b[0] = a[4] * a[8] - a[5] * a[7];
    b[3] = a[5] * a[6] - a[3] * a[8];
    b[6] = a[3] * a[7] - a[4] * a[6];
    b[1] = a[2] * a[7] - a[1] * a[8];
    b[4] = a[0] * a[8] - a[2] * a[6];
    b[7] = a[1] * a[6] - a[0] * a[7];
    b[2] = a[1] * a[5] - a[2] * a[4];
    b[5] = a[2] * a[3] - a[0] * a[5];
    b[8] = a[0] * a[4] - a[1] * a[3];
    double r = 1.0 / dt;
    for (int k = 0; k < 9; ++k) o[k] = b[k] * r;
}
static inline void mv3(const double *A, const double *v, double *o) {
    for (int i = 0; i < 3; ++i) o[i] = A[3 * i] * v[0] + A[3 * i + 1] * v[1] + A[3 * i + 2] * v[2];
}
static inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
/* rigid_reduce_kernel, affine.py:456-473 */
static void rigid_reduce(d2o_solver *s) {
    for (int b = 0; b < s->n_rig; ++b) {
        int e = s->r_env[b];
        double Hi[9], y[3], z[3], zy[3];
        inv3(s->r_Hc + 9 * b, Hi);
        const double *g = s->r_gq + 3 * b, *gp = s->r_gq_prev + 3 * b;
        for (int r = 0; r < 3; ++r) y[r] = g[r] - gp[r];
        mv3(Hi, g, z); mv3(Hi, y, zy);
        s->gPg[e] += dot3(g, z);
        s->g_Py[e] += dot3(g, zy);
        s->y_Py[e] += dot3(y, zy);
        memcpy(s->r_zq + 3 * b, z, sizeof z);
    }
}
/* rigid_direction_kernel, affine.py:476-486 */
static void rigid_direction(d2o_solver *s) {
    for (int k = 0; k < s->n_rign; ++k) {
        int b = s->r_grp[k], i = s->r_node[k];
        const double *z = s->r_zq + 3 * b;
        v2 rr = arm(ld(s->x, i), s->r_acc + 3 * b);
        st(s->p, i, sub(ld(s->p, i), V(z[0] - z[2] * rr.y, z[1] + z[2] * rr.x)));
    }
}

/* ------------------------------------------------------------------ Dai-Kou direction, kernels.py:160-230 */
static void mask_grad(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i) st(s->grad, i, cw(ld(s->grad, i), ld(s->free_, i)));
}
static void dk_reduce(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i) {
        int e = s->node2env[i];
        v2 dh = ld(s->diagH, i), fr = ld(s->free_, i);
        double Px = fr.x / fmax_(dh.x, 1.0e-12);
        double Py_ = fr.y / fmax_(dh.y, 1.0e-12);
        v2 g = ld(s->grad, i), pp = ld(s->p, i);
        v2 yy = sub(g, ld(s->grad_prev, i));
        double Pg0 = Px * g.x, Pg1 = Py_ * g.y;
        double Py0 = Px * yy.x, Py1 = Py_ * yy.y;
        s->gPg[e] += g.x * Pg0 + g.y * Pg1;
        s->g_p[e] += g.x * pp.x + g.y * pp.y;
        s->g_Py[e] += g.x * Py0 + g.y * Py1;
        s->y_p[e] += yy.x * pp.x + yy.y * pp.y;
        s->y_Py[e] += yy.x * Py0 + yy.y * Py1;
    }
}
static void finalize_beta(d2o_solver *s, int it) {
    for (int e = 0; e < s->B; ++e) {
        double b = 0.0;
        if (it > 0) {
            double ytp = s->y_p[e];
            if (fabs_(ytp) > 1.0e-30) b = s->g_Py[e] / ytp - s->y_Py[e] * s->g_p[e] / (ytp * ytp);
        }
        double t = -s->gPg[e] + b * s->g_p[e];
        if (t >= 0.0) { b = 0.0; t = -s->gPg[e]; }
        s->beta[e] = b; s->gTp[e] = t;
    }
}
/* cg_guard_kernel, solver.py:76-94 */
static void cg_guard(d2o_solver *s, const double *hold) {
    for (int e = 0; e < s->B; ++e)
        if (hold[e] <= 0.0 && s->y_p[e] < s->cg_guard * s->alpha[e] * s->pHp[e]) {
            s->beta[e] = 0.0; s->gTp[e] = -s->gPg[e];
        }
}
static void update_p(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i) {
        int e = s->node2env[i];
        v2 dh = ld(s->diagH, i), fr = ld(s->free_, i), g = ld(s->grad, i), pi = ld(s->p, i);
        double bb = s->beta[e];
        double px = -fr.x / fmax_(dh.x, 1.0e-12) * g.x + bb * pi.x;
        double py = -fr.y / fmax_(dh.y, 1.0e-12) * g.y + bb * pi.y;
        st(s->p, i, cw(V(px, py), fr));
    }
}

/* ------------------------------------------------------------------ curvature, kernels.py:234-299 */
static void pHp_reset(d2o_solver *s) {
    for (int e = 0; e < s->B; ++e) {
        s->pHp[e] = 0.0; s->alpha[e] = s->alpha_max; s->p_inf[e] = 0.0; s->clr_min[e] = BIG;
    }
}
static void pHp_mass(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i) {
        int e = s->node2env[i];
        v2 pp = ld(s->p, i);
        s->pHp[e] += s->mass[i] * (pp.x * pp.x + pp.y * pp.y);
        amax(s->p_inf, e, len(pp));
    }
}
static void pHp_elastic(d2o_solver *s) {
    for (int t = 0; t < s->T; ++t) {
        int i0 = s->tri[3 * t], i1 = s->tri[3 * t + 1], i2 = s->tri[3 * t + 2];
        m2 Bt = ldm(s->Bm, t);
        m2 F = mmul(ds_from_nodes(ld(s->x, i0), ld(s->x, i1), ld(s->x, i2)), Bt);
        double pe[6] = {s->p[2 * i0], s->p[2 * i0 + 1], s->p[2 * i1], s->p[2 * i1 + 1], s->p[2 * i2], s->p[2 * i2 + 1]};
        double val = s->area[t] * nh_pHp_elem(F, Bt, pe, s->mu[t], s->lam[t]);
        val = fmax_(val, 0.0);
        s->pHp[s->tri2env[t]] += s->h2 * val;
    }
}
static void pHp_disc(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b], e = s->b2e[b];
        v2 diff = sub(ld(s->x, n), V(c.cx, c.cy));
        double dc = len(diff), d = dc - c.r;
        amin(s->clr_min, e, d);
        if (d <= 0.0 || d >= s->dhat) continue;
        v2 nh = vdiv(diff, dc), pp = ld(s->p, n);
        double pn = dot(pp, nh);
        v2 pt = sub(pp, scl(pn, nh));
        double bp = barrier_bp(d, s->dhat), bpp = barrier_bpp(d, s->dhat);
        double val = s->kappa * (bpp * pn * pn + (bp / dc) * dot(pt, pt));
        val = fmax_(val, 0.0);
        s->pHp[e] += s->h2 * val;
    }
}
/* pHp_sdf_kernel, core/sdf.py:157-171 */
static void pHp_sdf(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b], e = s->b2e[b];
        sdfhit h = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, ld(s->x, n));
        amin(s->clr_min, e, h.d);
        if (h.d <= 0.0 || h.d >= s->dhat) continue;
        v2 pp = ld(s->p, n);
        double gp = dot(h.g, pp);
        double val = s->kappa * (barrier_bpp(h.d, s->dhat) * gp * gp + barrier_bp(h.d, s->dhat) * dot(pp, mvec(h.H, pp)));
        val = fmax_(val, 0.0);
        s->pHp[e] += s->h2 * val;
    }
}
/* pHp_friction_disc_kernel, kernels.py:684-711 */
static void pHp_friction_disc(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        v2 fr = ld(s->free_, n);
        if (fr.x <= 0.5 && fr.y <= 0.5) continue;
        v2 diff = sub(ld(s->x, n), V(c.cx, c.cy));
        double dc = len(diff), d = dc - c.r;
        if (d <= 0.0 || d >= s->dhat) continue;
        v2 nh = vdiv(diff, dc);
        double f_n = s->kappa * fabs_(barrier_bp(d, s->dhat));
        v2 v = vsc(sub(ld(s->x, n), ld(s->xn, n)), s->inv_dt);
        v2 vt = sub(v, scl(dot(v, nh), nh));
        double kt = s->h2 * c.mu * f_n * s->inv_dt / fmax_(len(vt), s->epsv);
        v2 th = V(-nh.y, nh.x);
        double pt = dot(cw(ld(s->p, n), fr), th);
        s->pHp[s->b2e[b]] += kt * pt * pt;
    }
}
/* pHp_friction_sdf_kernel, core/sdf.py:236-255 */
static void pHp_friction_sdf(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        v2 fr = ld(s->free_, n);
        if (fr.x <= 0.5 && fr.y <= 0.5) continue;
        sdfhit h = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, ld(s->x, n));
        if (h.d <= 0.0 || h.d >= s->dhat) continue;
        double f_n, vtm; v2 nh, vt;
        sdf_fric_frame(h, ld(s->x, n), ld(s->xn, n), s->kappa, s->dhat, s->inv_dt, &f_n, &nh, &vt, &vtm);
        double kt = s->h2 * c.mu * f_n * s->inv_dt / fmax_(vtm, s->epsv);
        v2 th = V(-nh.y, nh.x);
        double pt = dot(cw(ld(s->p, n), fr), th);
        s->pHp[s->b2e[b]] += kt * pt * pt;
    }
}

/* ------------------------------------------------------------------ step caps, kernels.py:303-371 */
static void inversion_alpha(d2o_solver *s) {
    for (int t = 0; t < s->T; ++t) {
        int i0 = s->tri[3 * t], i1 = s->tri[3 * t + 1], i2 = s->tri[3 * t + 2];
        v2 e1 = sub(ld(s->x, i1), ld(s->x, i0)), e2 = sub(ld(s->x, i2), ld(s->x, i0));
        v2 q1 = sub(ld(s->p, i1), ld(s->p, i0)), q2 = sub(ld(s->p, i2), ld(s->p, i0));
        double a0 = cross2(e1, e2);
        double a1 = cross2(e1, q2) + cross2(q1, e2);
        double a2 = cross2(q1, q2);
        double target = s->area_shrink * a0;
        double cc = a0 - target;
        int e = s->tri2env[t];
        if (fabs_(a2) < 1.0e-24) {
            if (fabs_(a1) > 1.0e-24) {
                double sv = -cc / a1;
                if (sv > 0.0) amin(s->alpha, e, sv);
            }
            continue;
        }
        double disc = a1 * a1 - 4.0 * a2 * cc;
        if (disc < 0.0) continue;
        double sq = sqrt(disc);
        double r1 = (-a1 - sq) / (2.0 * a2), r2 = (-a1 + sq) / (2.0 * a2);
        double sv = BIG;
        if (r1 > 0.0) sv = fmin_(sv, r1);
        if (r2 > 0.0) sv = fmin_(sv, r2);
        if (sv < BIG) amin(s->alpha, e, sv);
    }
}
static void disc_ccd(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        v2 o = sub(ld(s->x, n), V(c.cx, c.cy)), d = ld(s->p, n);
        double a = dot(d, d);
        if (a < 1.0e-24) continue;
        double bq = 2.0 * dot(o, d);
        double cq = dot(o, o) - c.r * c.r;
        double disc = bq * bq - 4.0 * a * cq;
        if (disc < 0.0) continue;
        double sq = sqrt(disc);
        double r1 = (-bq - sq) / (2.0 * a), r2 = (-bq + sq) / (2.0 * a);
        double sv = BIG;
        if (r1 > 0.0) sv = fmin_(sv, r1);
        if (r2 > 0.0) sv = fmin_(sv, r2);
        if (sv < BIG) amin(s->alpha, s->b2e[b], s->ccd_eta * sv);
    }
}
/* sdf_ccd_kernel, core/sdf.py:297-306 */
static void sdf_ccd(d2o_solver *s, collider c) {
    for (int b = 0; b < s->Nb; ++b) {
        int n = s->bnd[b];
        sdfhit h = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, ld(s->x, n));
        double gp = dot(h.g, ld(s->p, n));
        if (gp >= 0.0 || h.d <= 0.0) continue;
        amin(s->alpha, s->b2e[b], s->ccd_eta * h.d / (-gp));
    }
}
/* alpha_finalize_kernel, kernels.py:374-423 (+ the optional relative gradient-norm test) */
static void alpha_finalize(d2o_solver *s, int it, const double *gn2) {
    for (int e = 0; e < s->B; ++e) {
        if (s->active[e] == 0) continue;
        if (s->gtol > 0.0) {
            if (it == 0) s->gn0[e] = gn2[e];
            else if (gn2[e] <= s->gtol * s->gtol * s->gn0[e]) { s->active[e] = 0; continue; }
        }
        double ph = s->pHp[e];
        double a = s->alpha[e];
        if (ph > 0.0) a = fmin_(a, -s->gTp[e] / ph);
        if (s->clr_min[e] < s->near_factor * s->dhat && s->p_inf[e] > 0.0) a = fmin_(a, 0.5 * s->dhat / s->p_inf[e]);
        if (a <= 0.0) { s->active[e] = 0; s->alpha[e] = 0.0; continue; }
        s->alpha[e] = a;
        if (s->tol_x > 0.0 && a * s->p_inf[e] < s->tol_x) { s->active[e] = 0; s->iters[e] += 1; continue; }
        double d = -a * s->gTp[e] - 0.5 * a * a * ph;
        s->dE[e] = d;
        if (it == 0) s->dE0[e] = fmax_(d, 1.0e-300);
        else if (d < s->eps * s->dE0[e]) s->active[e] = 0;
        s->iters[e] += 1;
    }
}
static void update_x(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i) {
        int e = s->node2env[i];
        if (s->active[e] == 0) continue;
        st(s->x, i, add(ld(s->x, i), scl(s->alpha[e], ld(s->p, i))));
    }
}
static void set_x_from_x0(d2o_solver *s) {
    for (int i = 0; i < s->N; ++i) {
        int e = s->node2env[i];
        if (s->active[e] == 0) continue;
        st(s->x, i, add(ld(s->x0buf, i), scl(s->alpha[e], ld(s->p, i))));
    }
}

/* ------------------------------------------------------------------ energy, solver.py:453-498 */
/* The collider level set at n points (test access): sdf_eval(...).d, or |x - c| - r for a
   disc (kind 0, radius rx). */
void d2o_sdf(int kind, double cx, double cy, double rx, double ry, double rref, const double *pts, int n,
             double *d) {
    for (int i = 0; i < n; ++i) {
        v2 x = ld(pts, i);
        d[i] = kind == 0 ? len(sub(x, V(cx, cy))) - rx : sdf_eval(kind, cx, cy, rx, ry, rref, x).d;
    }
}

/* sdf_eval with its gradient (n x 2) and Hessian (n x 4, row-major) at each point, for the
   adjoint oracle's collider tangent (chvp_sdf_kernel, implicit/adjoint.py:101-114) */
void d2o_sdf_full(int kind, double cx, double cy, double rx, double ry, double rref, const double *pts, int n,
                  double *d, double *g, double *H) {
    for (int i = 0; i < n; ++i) {
        sdfhit h = sdf_eval(kind, cx, cy, rx, ry, rref, ld(pts, i));
        d[i] = h.d;
        g[2 * i] = h.g.x; g[2 * i + 1] = h.g.y;
        H[4 * i] = h.H.a; H[4 * i + 1] = h.H.b; H[4 * i + 2] = h.H.c; H[4 * i + 3] = h.H.d;
    }
}

/* ------------------------------------------------------------------ Springs, implicit/actuation.py:381-476 */
typedef struct { double ten, kt, len; v2 n; } spring_at_t;
/* _spring (:396-402): tension k (|d| - L0), tangential stiffness max(k (1 - L0/|d|), 0) */
static spring_at_t spring_at(const d2o_solver *s, int k) {
    int a = s->sp_a[k], b = s->sp_b[k];
    v2 xb = b >= 0 ? ld(s->x, b) : ld(s->sp_anchor, k);
    v2 d = sub(ld(s->x, a), xb);
    double ln = sqrt(dot(d, d) + 1.0e-30);
    spring_at_t r;
    r.ten = s->sp_k[k] * (ln - s->sp_L0[k]);
    r.kt = fmax_(s->sp_k[k] * (1.0 - s->sp_L0[k] / ln), 0.0);
    r.len = ln;
    r.n = vdiv(d, ln);
    return r;
}
static void spring_grad(d2o_solver *s) {  /* grad_diag_spring_kernel, :405-424 */
    for (int k = 0; k < s->n_spring; ++k) {
        spring_at_t r = spring_at(s, k);
        int a = s->sp_a[k], b = s->sp_b[k];
        double kk = s->sp_k[k];
        v2 g = scl(s->h2 * r.ten, r.n);
        v2 hd = V(s->h2 * (kk * r.n.x * r.n.x + r.kt * (1.0 - r.n.x * r.n.x)),
                  s->h2 * (kk * r.n.y * r.n.y + r.kt * (1.0 - r.n.y * r.n.y)));
        atomic_add2(s->grad, a, g);
        atomic_add2(s->diagH, a, hd);
        if (b >= 0) {
            atomic_add2(s->grad, b, scl(-1.0, g));
            atomic_add2(s->diagH, b, hd);
        }
    }
}
static void spring_pHp(d2o_solver *s) {  /* pHp_spring_kernel, :427-444 */
    for (int k = 0; k < s->n_spring; ++k) {
        spring_at_t r = spring_at(s, k);
        int a = s->sp_a[k], b = s->sp_b[k];
        v2 dp = ld(s->p, a);
        if (b >= 0) dp = sub(dp, ld(s->p, b));
        double along = dot(dp, r.n);
        s->pHp[s->sp2env[k]] += s->h2 * (s->sp_k[k] * along * along + r.kt * (dot(dp, dp) - along * along));
    }
}
static void spring_energy(d2o_solver *s, double *E) {  /* energy_spring_kernel, :447-456 */
    for (int k = 0; k < s->n_spring; ++k) {
        spring_at_t r = spring_at(s, k);
        double ext = r.len - s->sp_L0[k];
        E[s->sp2env[k]] += 0.5 * s->h2 * s->sp_k[k] * ext * ext;
    }
}
/* ------------------------------------------------------------------ Pressure, implicit/actuation.py:80-152 */
static void pressure_grad(d2o_solver *s) {  /* grad_pressure_kernel, :98-108 */
    for (int e = 0; e < s->n_pedge; ++e) {
        int a = s->pe_a[e], b = s->pe_b[e];
        v2 t = sub(ld(s->x, b), ld(s->x, a));
        v2 g = scl(-0.5 * s->h2 * s->ch_p[s->pe_ch[e]], V(t.y, -t.x));
        atomic_add2(s->grad, a, g);
        atomic_add2(s->grad, b, g);
    }
}
static void pressure_pHp(d2o_solver *s) {  /* pHp_pressure_kernel, :111-118 */
    for (int e = 0; e < s->n_pedge; ++e) {
        int c = s->pe_ch[e];
        v2 pa = ld(s->p, s->pe_a[e]), pb = ld(s->p, s->pe_b[e]);
        s->pHp[s->ch2env[c]] += -s->h2 * s->ch_p[c] * (pa.x * pb.y - pa.y * pb.x);
    }
}
static void pressure_energy(d2o_solver *s, double *E) {  /* energy_pressure_kernel, :121-130 */
    for (int e = 0; e < s->n_pedge; ++e) {
        int c = s->pe_ch[e];
        v2 ref = ld(s->ch_ref, c);
        v2 ra = sub(ld(s->x, s->pe_a[e]), ref), rb = sub(ld(s->x, s->pe_b[e]), ref);
        E[s->ch2env[c]] += -s->h2 * s->ch_p[c] * 0.5 * (ra.x * rb.y - ra.y * rb.x);
    }
}

static void energy_into(d2o_solver *s, double *E) {
    for (int e = 0; e < s->B; ++e) E[e] = 0.0;
    for (int i = 0; i < s->N; ++i) {  /* energy_kernel, kernels.py:445-452 */
        v2 d = sub(ld(s->x, i), ld(s->xhat, i));
        E[s->node2env[i]] += 0.5 * s->mass[i] * (d.x * d.x + d.y * d.y);
    }
    for (int t = 0; t < s->T; ++t) {  /* energy_elastic_kernel, kernels.py:455-468 */
        int i0 = s->tri[3 * t], i1 = s->tri[3 * t + 1], i2 = s->tri[3 * t + 2];
        m2 F = mmul(ds_from_nodes(ld(s->x, i0), ld(s->x, i1), ld(s->x, i2)), ldm(s->Bm, t));
        double J = det2(F);
        double logJ = log(fmax_(J, 1.0e-6));
        double I2 = ddot(F, F);
        double psi = 0.5 * s->mu[t] * (I2 - 2.0) - s->mu[t] * logJ + 0.5 * s->lam[t] * logJ * logJ;
        E[s->tri2env[t]] += s->h2 * s->area[t] * psi;
    }
    for (int k = 0; k < s->n_col; ++k) {
        collider c = col_at(s, k);
        for (int b = 0; b < s->Nb; ++b) {
            double d;
            if (c.kind == 0) d = len(sub(ld(s->x, s->bnd[b]), V(c.cx, c.cy))) - c.r;
            else d = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, ld(s->x, s->bnd[b])).d;
            if (d <= 0.0 || d >= s->dhat) continue;
            E[s->b2e[b]] += s->h2 * s->kappa * barrier_b(d, s->dhat);
        }
    }
    if (s->friction) {
        for (int k = 0; k < s->n_col; ++k) {
            collider c = col_at(s, k);
            for (int b = 0; b < s->Nb; ++b) {
                int n = s->bnd[b];
                v2 fr = ld(s->free_, n);
                if (fr.x <= 0.5 && fr.y <= 0.5) continue;
                if (c.kind == 0) {  /* energy_friction_disc_kernel, kernels.py:483-513 */
                    v2 diff = sub(ld(s->x, n), V(c.cx, c.cy));
                    double dc = len(diff), d = dc - c.r;
                    if (d <= 0.0 || d >= s->dhat) continue;
                    v2 nh = vdiv(diff, dc);
                    double f_n = s->kappa * fabs_(barrier_bp(d, s->dhat));
                    v2 v = vsc(sub(ld(s->x, n), ld(s->xn, n)), s->inv_dt);
                    v2 vt = sub(v, scl(dot(v, nh), nh));
                    double ut = len(vt) / s->inv_dt;
                    double a = s->epsv / s->inv_dt;
                    double f0 = ut - a * 0.5;
                    if (ut < a) f0 = ut * ut / (2.0 * a);
                    E[s->b2e[b]] += s->h2 * c.mu * f_n * f0;
                } else {  /* energy_friction_sdf_kernel, core/sdf.py:274-294 */
                    sdfhit h = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, ld(s->x, n));
                    if (h.d <= 0.0 || h.d >= s->dhat) continue;
                    double f_n, vtm; v2 nh, vt;
                    sdf_fric_frame(h, ld(s->x, n), ld(s->xn, n), s->kappa, s->dhat, s->inv_dt, &f_n, &nh, &vt, &vtm);
                    double ut = vtm / s->inv_dt;
                    double a = s->epsv / s->inv_dt;
                    double f0 = ut - a * 0.5;
                    if (ut < a) f0 = ut * ut / (2.0 * a);
                    E[s->b2e[b]] += s->h2 * c.mu * f_n * f0;
                }
            }
        }
    }
    /* terms in the reference's order (implicit/integrator.py:151-229): ExternalForce,
       AffineBodies, IPCContact, Springs, Pressure, Tendon */
    if (s->has_ext) ext_energy(s, E);
    if (s->n_aff) affine_energy(s, E);
    if (s->has_ipc) { ipc_launch L = ipc_base(s, 2, s->p, E, s->clr_min, s->alpha); ipc_pair(&L); }
    if (s->n_spring) spring_energy(s, E);
    if (s->n_pedge) pressure_energy(s, E);
    if (s->n_tendon) tendon_energy(s, E);
}
void d2o_energy(d2o_solver *s, double *buf) { energy_into(s, buf); }
/* the IPC contact term alone (IPCContact.energy, ipc_contact.py:414-429): barrier and lagged
   friction between bodies at s->x, friction slip measured from s->xn; per environment */
void d2o_ipc_energy(d2o_solver *s, double *buf) {
    for (int e = 0; e < s->B; ++e) buf[e] = 0.0;
    if (!s->has_ipc) return;
    ipc_launch L = ipc_base(s, 2, s->p, buf, s->clr_min, s->alpha);
    ipc_pair(&L);
}

/* One term alone at s->x (which: 0 Springs, 1 Pressure, 2 IPC contact between bodies): its
   gradient and diagonal into s->grad / s->diagH and its curvature along s->p into s->pHp (all
   zeroed first), its energy per environment into E — the derivative checks of
   tests/test_actuation.py and tests/test_ipc.py. For IPC the friction slip is measured from
   s->xn, and the step caps its curvature pass also computes go to scratch. */
void d2o_term(d2o_solver *s, int which, double *E) {
    memset(s->grad, 0, sizeof(double) * 2 * s->N);
    memset(s->diagH, 0, sizeof(double) * 2 * s->N);
    for (int e = 0; e < s->B; ++e) { s->pHp[e] = 0.0; E[e] = 0.0; }
    if (which == 0) { spring_grad(s); spring_pHp(s); spring_energy(s, E); }
    else if (which == 1) { pressure_grad(s); pressure_pHp(s); pressure_energy(s, E); }
    else if (s->has_ipc) {
        double *a = (double *)malloc(sizeof(double) * (size_t)s->B);
        double *c = (double *)malloc(sizeof(double) * (size_t)s->B);
        for (int e = 0; e < s->B; ++e) { a[e] = 3.0; c[e] = 1.0e30; }
        ipc_launch L0 = ipc_base(s, 0, s->p, E, c, a);
        ipc_pair(&L0);
        ipc_launch L1 = ipc_base(s, 1, s->p, E, c, a);
        ipc_pair(&L1);
        ipc_launch L2 = ipc_base(s, 2, s->p, E, c, a);
        ipc_pair(&L2);
        free(a);
        free(c);
    }
}

/* ------------------------------------------------------------------ the loop, solver.py:252-425 */
static void iterate(d2o_solver *s) {
    double *zeroB = (double *)calloc((size_t)s->B, sizeof(double));
    double *gn2 = (double *)calloc((size_t)s->B, sizeof(double));
    for (int it = 0; it < s->iter_max; ++it) {
        if (s->has_ipc && s->pending) {  /* IPCContact.before_iteration, ipc_contact.py:475-483 */
            ipc_sweep(s);
            for (int e = 0; e < s->B; ++e) if (s->q_inf[e] > 0.0) s->active[e] = 1;
            if (it % 8 == 7) s->pending = !all_beta_done(s);
        }
        if (s->conv_check && it && it % s->conv_check == 0) {
            int any = 0;
            for (int e = 0; e < s->B; ++e) any += s->active[e];
            if (any == 0) break;
        }
        grad_diag_mass(s);
        grad_diag_elastic(s);
        if (s->n_rig) memcpy(s->diag_el, s->diagH, sizeof(double) * 2 * s->N);  /* RigidModes.after_elastic */
        for (int k = 0; k < s->n_col; ++k) {
            collider c = col_at(s, k);
            if (c.kind == 0) grad_diag_disc(s, c); else if (c.kind > 0) grad_diag_sdf(s, c);
        }
        if (s->friction)
            for (int k = 0; k < s->n_col; ++k) {
                collider c = col_at(s, k);
                if (c.kind == 0) grad_friction_disc(s, c); else if (c.kind > 0) grad_friction_sdf(s, c);
            }
        if (s->has_ext) ext_grad(s);
        if (s->has_ipc) { ipc_launch L = ipc_base(s, 0, s->p, s->Ener, s->clr_min, s->alpha); ipc_pair(&L); }
        if (s->n_spring) spring_grad(s);
        if (s->n_pedge) pressure_grad(s);
        if (s->n_tendon) tendon_grad(s);
        if (s->n_aff) affine_gather(s);
        if (s->n_rig) rigid_gather(s);
        mask_grad(s);

        for (int e = 0; e < s->B; ++e) { s->gPg[e] = 0; s->g_p[e] = 0; s->g_Py[e] = 0; s->y_p[e] = 0; s->y_Py[e] = 0; }
        dk_reduce(s);
        if (s->n_aff) affine_reduce(s);
        if (s->n_rig) rigid_reduce(s);
        finalize_beta(s, it);
        if (s->cg_guard > 0.0 && it > 0)
            cg_guard(s, (s->has_ipc && s->pending) ? s->q_inf : zeroB);
        update_p(s);
        if (s->n_aff) affine_direction(s);
        if (s->n_rig) rigid_direction(s);

        pHp_reset(s);
        pHp_mass(s);
        pHp_elastic(s);
        for (int k = 0; k < s->n_col; ++k) {
            collider c = col_at(s, k);
            if (c.kind == 0) pHp_disc(s, c); else if (c.kind > 0) pHp_sdf(s, c);
        }
        if (s->friction)
            for (int k = 0; k < s->n_col; ++k) {
                collider c = col_at(s, k);
                if (c.kind == 0) pHp_friction_disc(s, c); else if (c.kind > 0) pHp_friction_sdf(s, c);
            }
        if (s->n_aff) affine_pHp(s);
        if (s->has_ipc) {
            for (int e = 0; e < s->B; ++e) s->clr[e] = 1.0e30;
            ipc_launch L = ipc_base(s, 1, s->p, s->Ener, s->clr, s->alpha);
            ipc_pair(&L);
            ipc_far_cap(s, s->p_inf, s->alpha);
        }
        if (s->n_spring) spring_pHp(s);
        if (s->n_pedge) pressure_pHp(s);
        if (s->n_tendon) tendon_pHp(s);
        inversion_alpha(s);
        for (int k = 0; k < s->n_col; ++k) {
            collider c = col_at(s, k);
            if (c.kind == 0) disc_ccd(s, c); else if (c.kind > 0) sdf_ccd(s, c);
        }
        if (s->gtol > 0.0) {
            for (int e = 0; e < s->B; ++e) gn2[e] = 0.0;
            for (int i = 0; i < s->N; ++i) {
                v2 g = ld(s->grad, i);
                gn2[s->node2env[i]] += g.x * g.x + g.y * g.y;
            }
        }
        alpha_finalize(s, it, gn2);
        if (!s->line_search) {
            update_x(s);
            if (s->n_aff) affine_advance(s);
        } else {
            energy_into(s, s->Els_prev);
            memcpy(s->x0buf, s->x, sizeof(double) * 2 * s->N);
            if (s->n_aff) memcpy(s->a_q0, s->a_q, sizeof(double) * 6 * s->n_aff);
            for (int bt = 0; bt < s->n_bt; ++bt) {
                set_x_from_x0(s);
                if (s->n_aff) affine_trial(s);
                energy_into(s, s->Ener);
                for (int e = 0; e < s->B; ++e) {  /* ls_halve_kernel, solver.py:63-73 */
                    if (s->active[e] == 0) continue;
                    if (s->Ener[e] > s->Els_prev[e] + s->ls_tol * (fabs_(s->Els_prev[e]) + 1.0)) s->alpha[e] = s->alpha[e] * 0.5;
                }
            }
            set_x_from_x0(s);
            if (s->n_aff) affine_trial(s);
        }
    }
    free(zeroB);
    free(gn2);
}

/* PNCG2DSolver.step_targets, solver.py:433-451 */
int d2o_step(d2o_solver *s) {
    init_step(s);
    if (!s->has_ipc) apply_bc(s);
    else {  /* IPCContact.advance_bc, ipc_contact.py:465-473 */
        s->pending = 0;
        if (s->n_bc) { ipc_sweep(s); s->pending = !all_beta_done(s); }
    }
    for (int e = 0; e < s->B; ++e) { s->dE0[e] = 0.0; s->active[e] = 1; s->iters[e] = 0; }
    memset(s->p, 0, sizeof(double) * 2 * s->N);
    memset(s->grad, 0, sizeof(double) * 2 * s->N);
    iterate(s);
    for (int i = 0; i < s->N; ++i)  /* commit_v_kernel, kernels.py:437-441 */
        st(s->v, i, vsc(sub(ld(s->x, i), ld(s->xn, i)), 1.0 / s->dt));
    return 0;
}
