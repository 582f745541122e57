// Device math shared by the step kernels: collider signed distances, the IPC log barrier,
// the node-to-segment helpers and the 6x6 affine-block algebra.
//
// Formulas follow the reference (core/math.py, core/sdf.py, implicit/ipc_contact.py,
// implicit/affine.py; lines cited per function). The element routines of the step kernel
// use closed forms that are algebraically equal to the reference's directional second
// derivatives but cost a fraction of the FP64 operations (see pncg_step.cu).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace d2f {

// Barriers of the thread group working on one scene. Both use the non-aligned PTX forms,
// which count every thread on its own: a warp whose lanes arrive at different times (after
// loops whose trip counts differ lane by lane) is waited for in full. The aligned block
// barrier that __syncthreads() emits let warps through before slower warps of the same
// block had arrived on this GB300 build (measured: up to 3e5 cycles of skew after a loop of
// uneven trip counts), after which block reductions read shared values of another phase;
// these kernels therefore never use it.
__device__ __forceinline__ void block_barrier() { asm volatile("barrier.sync 0;" ::: "memory"); }
// The whole thread-block cluster: arrive (release) and wait (acquire), non-aligned.
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dabs(double a) { return a >= 0.0 ? a : -a; }

template <class R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <class R> __device__ __forceinline__ R rabs(R a) { return a >= R(0) ? a : -a; }
template <class R> __device__ __forceinline__ R rlog(R a);
template <> __device__ __forceinline__ double rlog<double>(double a) { return log(a); }
template <> __device__ __forceinline__ float rlog<float>(float a) { return logf(a); }
template <class R> __device__ __forceinline__ R rsqrt_(R a);
template <> __device__ __forceinline__ double rsqrt_<double>(double a) { return sqrt(a); }
template <> __device__ __forceinline__ float rsqrt_<float>(float a) { return sqrtf(a); }

// ---- IPC log barrier b(d) = -(d - dhat)^2 log(d / dhat) and its derivatives, core/math.py:112-129
template <class R> __device__ __forceinline__ R barrier_b(R d, R dhat) {
    R u = d - dhat;
    return -(u * u) * rlog<R>(d / dhat);
}
template <class R> __device__ __forceinline__ R barrier_bp(R d, R dhat) {
    R u = d - dhat;
    return R(-2) * u * rlog<R>(d / dhat) - (u * u) / d;
}
template <class R> __device__ __forceinline__ R barrier_bpp(R d, R dhat) {
    R u = d - dhat;
    return R(-2) * rlog<R>(d / dhat) - R(4) * u / d + (u * u) / (d * d);
}

// ---- collider signed distance, core/sdf.py:44-137. Evaluated in FP64 (positions are FP64).
struct SdfHit {
    double d, gx, gy, H00, H01, H10, H11;
};

__device__ __forceinline__ double seg_closest(double px, double py, double ax, double ay, double bx,
                                              double by, double &qx, double &qy, double &isv) {
    double abx = bx - ax, aby = by - ay;
    double t = ((px - ax) * abx + (py - ay) * aby) / dmax(abx * abx + aby * aby, 1.0e-30);
    double tc = dmin(dmax(t, 0.0), 1.0);
    qx = ax + tc * abx;
    qy = ay + tc * aby;
    isv = (t <= 0.0 || t >= 1.0) ? 1.0 : 0.0;
    double dx = px - qx, dy = py - qy;
    return sqrt(dx * dx + dy * dy);
}

// kinds: 0 disc, 1 ellipse, 2 rounded box, 3 rounded triangle, 4 half-space
static __device__ __noinline__ SdfHit sdf_eval(int kind, double cx, double cy, double rx, double ry, double rref,
                                  double x, double y) {
    SdfHit h{0, 0, 0, 0, 0, 0, 0};
    if (kind == 4) {  // half-space: phi = n . (x - c), flat
        h.d = rx * (x - cx) + ry * (y - cy);
        h.gx = rx;
        h.gy = ry;
        return h;
    }
    if (kind == 0) {
        double dx = x - cx, dy = y - cy, dc = sqrt(dx * dx + dy * dy);
        double nx = dx / dc, ny = dy / dc, r = 1.0 / dc;
        h.d = dc - rx;
        h.gx = nx;
        h.gy = ny;
        h.H00 = (1.0 - nx * nx) * r;
        h.H01 = (0.0 - nx * ny) * r;
        h.H10 = (0.0 - ny * nx) * r;
        h.H11 = (1.0 - ny * ny) * r;
        return h;
    }
    if (kind == 1) {  // ellipse level set
        double ux = (x - cx) / rx, uy = (y - cy) / ry;
        double u = ux * ux + uy * uy, su = sqrt(dmax(u, 1.0e-18));
        double wx = (x - cx) / (rx * rx), wy = (y - cy) / (ry * ry);
        double f = rref / su, iu = 1.0 / u;
        h.d = rref * (su - 1.0);
        h.gx = f * wx;
        h.gy = f * wy;
        h.H00 = f * (1.0 / (rx * rx) - iu * (wx * wx));
        h.H01 = f * (0.0 - iu * (wx * wy));
        h.H10 = f * (0.0 - iu * (wy * wx));
        h.H11 = f * (1.0 / (ry * ry) - iu * (wy * wy));
        return h;
    }
    if (kind == 2) {  // rounded box
        double r = dmin(dmax(rref, 0.0), dmin(rx, ry));
        double sx = x < cx ? -1.0 : 1.0, sy = y < cy ? -1.0 : 1.0;
        double qx = sx * (x - cx) - (rx - r), qy = sy * (y - cy) - (ry - r);
        double mx = dmax(qx, 0.0), my = dmax(qy, 0.0);
        double ml = sqrt(mx * mx + my * my);
        h.d = ml + dmin(dmax(qx, qy), 0.0) - r;
        if (ml > 1.0e-12) {
            double gx = mx / ml, gy = my / ml;
            h.gx = sx * gx;
            h.gy = sy * gy;
            if (qx > 0.0 && qy > 0.0) {
                double off = -gx * gy / ml;
                h.H00 = gy * gy / ml;
                h.H01 = sx * sy * off;
                h.H10 = sx * sy * off;
                h.H11 = gx * gx / ml;
            }
        } else {
            if (qx > qy) { h.gx = sx; h.gy = 0.0; } else { h.gx = 0.0; h.gy = sy; }
        }
        return h;
    }
    // kind 3: rounded equilateral triangle, apex +y; rx = circumradius of the rounded shape
    double r3 = dmin(dmax(rref, 0.0), rx * 0.5), rin = rx - r3;
    const double c0 = 6.123233995736766e-17, s0 = 1.0;  // cos, sin of pi/2
    double c1 = cos(1.5707963267948966 + 2.0943951023931953), s1 = sin(1.5707963267948966 + 2.0943951023931953);
    double c2 = cos(1.5707963267948966 + 4.1887902047863905), s2 = sin(1.5707963267948966 + 4.1887902047863905);
    double v0x = cx + rin * c0, v0y = cy + rin * s0;
    double v1x = cx + rin * c1, v1y = cy + rin * s1;
    double v2x = cx + rin * c2, v2y = cy + rin * s2;
    double q0x, q0y, i0, q1x, q1y, i1, q2x, q2y, i2;
    double d0 = seg_closest(x, y, v0x, v0y, v1x, v1y, q0x, q0y, i0);
    double d1 = seg_closest(x, y, v1x, v1y, v2x, v2y, q1x, q1y, i1);
    double d2 = seg_closest(x, y, v2x, v2y, v0x, v0y, q2x, q2y, i2);
    double dm = d0, qmx = q0x, qmy = q0y, sm = i0;
    if (d1 < dm) { dm = d1; qmx = q1x; qmy = q1y; sm = i1; }
    if (d2 < dm) { dm = d2; qmx = q2x; qmy = q2y; sm = i2; }
    double k0 = (v1x - v0x) * (y - v0y) - (v1y - v0y) * (x - v0x);
    double k1 = (v2x - v1x) * (y - v1y) - (v2y - v1y) * (x - v1x);
    double k2 = (v0x - v2x) * (y - v2y) - (v0y - v2y) * (x - v2x);
    double sgn = (k0 >= 0.0 && k1 >= 0.0 && k2 >= 0.0) ? -1.0 : 1.0;
    double dl = dmax(dm, 1.0e-30);
    h.d = sgn * dm - r3;
    h.gx = (sgn / dl) * (x - qmx);
    h.gy = (sgn / dl) * (y - qmy);
    if (sm > 0.5 && sgn > 0.0) {
        double r = 1.0 / dl;
        h.H00 = (1.0 - h.gx * h.gx) * r;
        h.H01 = (0.0 - h.gx * h.gy) * r;
        h.H10 = (0.0 - h.gy * h.gx) * r;
        h.H11 = (1.0 - h.gy * h.gy) * r;
    }
    return h;
}

// ---- node-to-segment distance and additive CCD, implicit/ipc_contact.py:94-127 (FP64)
__device__ __forceinline__ double seg_dist(double px, double py, double ax, double ay, double bx, double by) {
    double abx = bx - ax, aby = by - ay;
    double t = ((px - ax) * abx + (py - ay) * aby) / dmax(abx * abx + aby * aby, 1.0e-30);
    t = dmin(dmax(t, 0.0), 1.0);
    double dx = (px - ax) - t * abx, dy = (py - ay) - t * aby;
    return sqrt(dx * dx + dy * dy);
}

__device__ inline double accd(double px, double py, double ax, double ay, double bx, double by,
                              double dpx, double dpy, double dax, double day, double dbx, double dby,
                              double g, double t_c) {
    double mx = (dpx + dax + dbx) / 3.0, my = (dpy + day + dby) / 3.0;
    dpx -= mx; dpy -= my; dax -= mx; day -= my; dbx -= mx; dby -= my;
    double lp = sqrt(dpx * dpx + dpy * dpy) + dmax(sqrt(dax * dax + day * day), sqrt(dbx * dbx + dby * dby));
    if (lp <= 1.0e-30) return t_c;
    double d = seg_dist(px, py, ax, ay, bx, by);
    double t = 0.0, tl = (d - g) / lp;
    for (int k = 0; k < 32; ++k) {
        double tn = t + tl;
        if (tn >= t_c) return t_c;
        d = seg_dist(px + tn * dpx, py + tn * dpy, ax + tn * dax, ay + tn * day, bx + tn * dbx, by + tn * dby);
        if (k > 0 && d < g) return t;
        t = tn;
        tl = 0.9 * d / lp;
    }
    return t;
}

// The ACCD advance of one pair run against an unbounded cap, summarised so that its result
// for ANY cap m <= t_c0 can be read off afterwards: accd(..., m) == (m <= T ? m : R).
// R is the return value with cap t_c0; T is the advance at which the loop stopped (the first
// step that would have crossed the gap, or the last one taken), +inf when it reached t_c0 or
// nothing moves. The reference reads the cap once per edge, after the edges before it have
// lowered it (ipc_contact.py:211, 241); this lets the caller replay that order exactly.
static __device__ __noinline__ double accd_profile(double px, double py, double ax, double ay, double bx, double by,
                                      double dpx, double dpy, double dax, double day, double dbx, double dby,
                                      double g, double t_c0, double &T) {
    double mx = (dpx + dax + dbx) / 3.0, my = (dpy + day + dby) / 3.0;
    dpx -= mx; dpy -= my; dax -= mx; day -= my; dbx -= mx; dby -= my;
    double lp = sqrt(dpx * dpx + dpy * dpy) + dmax(sqrt(dax * dax + day * day), sqrt(dbx * dbx + dby * dby));
    T = 1.0e300;
    if (lp <= 1.0e-30) return t_c0;
    double d = seg_dist(px, py, ax, ay, bx, by);
    double t = 0.0, tl = (d - g) / lp;
    for (int k = 0; k < 32; ++k) {
        double tn = t + tl;
        if (tn >= t_c0) return t_c0;
        d = seg_dist(px + tn * dpx, py + tn * dpy, ax + tn * dax, ay + tn * day, bx + tn * dbx, by + tn * dby);
        if (k > 0 && d < g) { T = tn; return t; }
        t = tn;
        tl = 0.9 * d / lp;
    }
    T = t;
    return t;
}

// The same profile in FP32, on the pair's geometry taken relative to one of its nodes (so
// the magnitudes are the pair's own, which FP32 resolves to ~1e-7 of them): the mixed step's
// step cap between bodies. The search ends 10 % short of each measured distance and stops at
// the margin g, which is far above that rounding. T = 3e38 when no contact within t_c0.
__device__ __forceinline__ float seg_dist_f(float px, float py, float ax, float ay, float bx, float by) {
    const float abx = bx - ax, aby = by - ay;
    float t = ((px - ax) * abx + (py - ay) * aby) / fmaxf(abx * abx + aby * aby, 1.0e-30f);
    t = fminf(fmaxf(t, 0.f), 1.f);
    const float dx = (px - ax) - t * abx, dy = (py - ay) - t * aby;
    return sqrtf(dx * dx + dy * dy);
}
static __device__ __noinline__ float accd_profile_f(float px, float py, float ax, float ay, float bx, float by,
                                                    float dpx, float dpy, float dax, float day, float dbx, float dby,
                                                    float g, float t_c0, float &T) {
    const float mx = (dpx + dax + dbx) / 3.f, my = (dpy + day + dby) / 3.f;
    dpx -= mx; dpy -= my; dax -= mx; day -= my; dbx -= mx; dby -= my;
    const float lp = sqrtf(dpx * dpx + dpy * dpy) + fmaxf(sqrtf(dax * dax + day * day), sqrtf(dbx * dbx + dby * dby));
    T = 3.0e38f;
    if (lp <= 1.0e-30f) return t_c0;
    float d = seg_dist_f(px, py, ax, ay, bx, by);
    float t = 0.f, tl = (d - g) / lp;
    for (int k = 0; k < 32; ++k) {
        const float tn = t + tl;
        if (tn >= t_c0) return t_c0;
        d = seg_dist_f(px + tn * dpx, py + tn * dpy, ax + tn * dax, ay + tn * day, bx + tn * dbx, by + tn * dby);
        if (k > 0 && d < g) { T = tn; return t; }
        t = tn;
        tl = 0.9f * d / lp;
    }
    T = t;
    return t;
}

// ---- Neo-Hookean on a 2x2 (FP64), core/math.py:75-93: used by the affine blocks
struct M2 { double a, b, c, d; };
__device__ __forceinline__ double det2(M2 A) { return A.a * A.d - A.c * A.b; }
__device__ __forceinline__ M2 nh_P(M2 F, double mu, double la) {
    double J = det2(F), logJ = log(dmax(J, 1.0e-6));
    double r = J != 0.0 ? 1.0 / J : 0.0;
    double c1 = la * logJ - mu;
    // F^-T = [[F11, -F10], [-F01, F00]] / J
    return M2{mu * F.a + c1 * (F.d * r), mu * F.b + c1 * (-F.c * r), mu * F.c + c1 * (-F.b * r),
              mu * F.d + c1 * (F.a * r)};
}
__device__ __forceinline__ M2 nh_d2(M2 F, M2 dF, double mu, double la) {
    double J = det2(F), logJ = log(dmax(J, 1.0e-6));
    double r = J != 0.0 ? 1.0 / J : 0.0;
    M2 G{F.d * r, -F.c * r, -F.b * r, F.a * r};
    double GdF = G.a * dF.a + G.b * dF.b + G.c * dF.c + G.d * dF.d;
    // G dF^T G
    M2 T{G.a * dF.a + G.b * dF.b, G.a * dF.c + G.b * dF.d, G.c * dF.a + G.d * dF.b, G.c * dF.c + G.d * dF.d};
    M2 GdFtG{T.a * G.a + T.b * G.c, T.a * G.b + T.b * G.d, T.c * G.a + T.d * G.c, T.c * G.b + T.d * G.d};
    double c1 = la * logJ - mu;
    return M2{mu * dF.a + la * GdF * G.a - c1 * GdFtG.a, mu * dF.b + la * GdF * G.b - c1 * GdFtG.b,
              mu * dF.c + la * GdF * G.c - c1 * GdFtG.c, mu * dF.d + la * GdF * G.d - c1 * GdFtG.d};
}
__device__ __forceinline__ double ddot2(M2 A, M2 B) { return A.a * B.a + A.b * B.b + A.c * B.c + A.d * B.d; }

// ---- 6x6 block: reduced Hessian, Cholesky with diagonal fallback, solve; affine.py:60-147
static __device__ __noinline__ void reduced_hessian(M2 A, double Mu, double La, double h2, const double *Hs, double (*H)[6]) {
    // Hs: x block then y block, 6 unique entries each: 00 01 02 11 12 22
    const int u[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) H[r][c] = 0.0;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            H[r][c] = Hs[u[r][c]];
            H[r + 3][c + 3] = Hs[6 + u[r][c]];
        }
    const int idx[4] = {1, 2, 4, 5};
    for (int k = 0; k < 4; ++k) {
        M2 E{k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0, k == 3 ? 1.0 : 0.0};
        M2 col = nh_d2(A, E, Mu, La);
        double cv[4] = {col.a, col.b, col.c, col.d};
        for (int r = 0; r < 4; ++r) H[idx[r]][idx[k]] += h2 * cv[r];
    }
    double a = A.a + A.d, b = A.c - A.b;
    double n = sqrt(a * a + b * b);
    if (n > 1.0e-12) {
        double f = 0.7071067811865476 / n;
        double t[4] = {-b * f, -a * f, a * f, -b * f};
        M2 Tm{t[0], t[1], t[2], t[3]};
        double lam_t = ddot2(Tm, nh_d2(A, Tm, Mu, La));
        if (lam_t < 0.0)
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) H[idx[r]][idx[c]] -= h2 * lam_t * t[r] * t[c];
    }
}

static __device__ __noinline__ void chol6(const double (*H)[6], double (*L)[6]) {
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) L[r][c] = 0.0;
    bool ok = true;
    for (int j = 0; j < 6; ++j) {
        double s = H[j][j];
        for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
        if (s <= 1.0e-9 * dabs(H[j][j]) || s <= 0.0) ok = false;
        if (ok) {
            double d = sqrt(s);
            L[j][j] = d;
            for (int i = j + 1; i < 6; ++i) {
                double v = H[i][j];
                for (int k = 0; k < j; ++k) v -= L[i][k] * L[j][k];
                L[i][j] = v / d;
            }
        }
    }
    if (!ok) {
        for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 6; ++c) L[r][c] = 0.0;
        for (int j = 0; j < 6; ++j) L[j][j] = sqrt(dmax(H[j][j], 1.0e-30));
    }
}

static __device__ __noinline__ void chol6_solve(const double (*L)[6], const double *b, double *x) {
    double y[6];
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[i][k] * y[k];
        y[i] = s / L[i][i];
    }
    for (int i = 5; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < 6; ++k) s -= L[k][i] * x[k];
        x[i] = s / L[i][i];
    }
}

}  // namespace d2f
