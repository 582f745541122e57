// adjoint.cu — the adjoint of the implicit step on the GPU: the linearised system of a
// converged step solved by preconditioned CG on the device, and the vector-Jacobian
// products to per-element stiffness and tendon tension.
//
// The reference (implicit/adjoint.py) solves, per checkpointed step k, backwards,
//     H_k lam_k = dJ/dx_k + (1 + drag) M lam_{k+1} - drag M lam_{k+2}        (:386-398)
// with H = M + h^2 (K_elastic + K_collider) on the free DOFs, the contact gate frozen at the
// converged x_k, by host MINRES whose every matrix-vector product crosses the host-device
// boundary twice (:224-246, :339-369). Here one thread block owns one scene and runs the
// whole Jacobi-preconditioned CG of that scene on the device, matrix-free: the element pass
// writes each corner's share of (K_elastic v), a node pass gathers it in ascending triangle
// order and adds inertia, the frozen collider barrier and the tendon's geometric stiffness.
// The tendon term is beyond the reference, which refuses tendons (:376-385).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "d2f_math.cuh"
#include "d2f_solver.h"
#include "pncg_kernel.cuh"

namespace d2f {
namespace adj {

constexpr int MAXC = 16;

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// the warp's sum in every lane (butterfly)
__device__ __forceinline__ double wsum_all(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// deterministic block sum of NV values (fixed tree), result to every thread
template <int NT, int NV>
__device__ __forceinline__ void bsum(double (&v)[NV], double *red) {
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const double t = wsum(v[k]);
        if (lane == 0) red[warp * NV + k] = t;
    }
    block_barrier();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = lane < NW ? red[lane * NV + k] : 0.0;
            t = wsum(t);
            if (lane == 0) red[NW * NV + k] = t;
        }
    }
    block_barrier();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = red[NW * NV + k];
    block_barrier();
}

// collider Hessian (2x2, frozen gate) and its clamped diagonal at x, for one boundary node
__device__ __forceinline__ void collider_hessian(const double *cd, int kind, double x, double y, double dhat,
                                                 double kappa, double &h00, double &h01, double &h11) {
    h00 = h01 = h11 = 0.0;
    double dd, nx, ny, H00 = 0, H01 = 0, H11 = 0;
    if (kind == 0) {
        const double ex = x - cd[1], ey = y - cd[2], dc = sqrt(ex * ex + ey * ey);
        dd = dc - cd[6];
        nx = ex / dc; ny = ey / dc;
        H00 = (1.0 - nx * nx) / dc; H01 = (0.0 - nx * ny) / dc; H11 = (1.0 - ny * ny) / dc;
    } else {
        const SdfHit h = sdf_eval(kind, cd[1], cd[2], cd[3], cd[4], cd[5], x, y);
        dd = h.d; nx = h.gx; ny = h.gy; H00 = h.H00; H01 = h.H01; H11 = h.H11;
    }
    if (dd <= 0.0 || dd >= dhat) return;
    const double bp = barrier_bp<double>(dd, dhat), bpp = barrier_bpp<double>(dd, dhat);
    // kappa (b'' g g^T + b' H_phi): chvp_disc_kernel / chvp_sdf_kernel (implicit/adjoint.py:87-114)
    h00 = kappa * (bpp * nx * nx + bp * H00);
    h01 = kappa * (bpp * nx * ny + bp * H01);
    h11 = kappa * (bpp * ny * ny + bp * H11);
}

// ---- contact between bodies (IPC), frictionless, active set frozen at x (ipc_pair_kernel
// terms, implicit/ipc_contact.py:174-296; the reference's adjoint refuses IPC)
// Index of (i, j), i <= j, in the upper triangle of a symmetric 6x6 stored row by row.
__device__ __forceinline__ int ut6(int i, int j) { return 6 * i - (i * (i - 1)) / 2 + (j - i); }

// The directional second derivative of the point-line distance |cross(ab, w)| / |ab| along
// v = (v_p, v_a, v_b): the same quadratic form in v as the step's curvature pass uses.
__device__ __forceinline__ double line_ddd(double abx, double aby, double wx, double wy, double Ll, double c0,
                                           const double *v) {
    const double dex = v[4] - v[2], dey = v[5] - v[3], dwx = v[0] - v[2], dwy = v[1] - v[3];
    const double c1 = (dex * wy - dey * wx) + (abx * dwy - aby * dwx);
    const double c2 = 2.0 * (dex * dwy - dey * dwx);
    const double L1 = (abx * dex + aby * dey) / Ll;
    const double Lq = ((dex * dex + dey * dey) - L1 * L1) / Ll;
    const double s0 = c0 / Ll, s1 = (c1 - s0 * L1) / Ll;
    const double ddd = (c2 - 2.0 * s1 * L1 - s0 * Lq) / Ll;
    return c0 < 0.0 ? -ddd : ddd;
}

// kappa (b''(d) g g^T + b'(d) grad^2 d) of one point-point term (the distance between the
// point and node `o` = 1 (a) or 2 (b)), times coef, added to the pair's block H.
__device__ __forceinline__ void point_block(double coef, double wx, double wy, double dist, double dhat, double kappa,
                                            int o, double *H) {
    const double nx = wx / dist, ny = wy / dist;
    const double bp = barrier_bp<double>(dist, dhat), bpp = barrier_bpp<double>(dist, dhat);
    const double K[2][2] = {{(1.0 - nx * nx) / dist, -nx * ny / dist}, {-nx * ny / dist, (1.0 - ny * ny) / dist}};
    const double n[2] = {nx, ny};
    const int dof[4] = {0, 1, 2 * o, 2 * o + 1};
    for (int r = 0; r < 4; ++r)
        for (int c = r; c < 4; ++c) {
            const double sr = r < 2 ? 1.0 : -1.0, sc = c < 2 ? 1.0 : -1.0;
            const double gg = sr * n[r & 1] * sc * n[c & 1];
            const double hd = sr * sc * K[r & 1][c & 1];
            H[ut6(dof[r], dof[c])] += coef * kappa * (bpp * gg + bp * hd);
        }
}

// Every barrier term of the node-edge pair (p, edge ge = (a, b)) at x, frozen: the edge
// interior with weights (1 - t, t), and each end with its vertex-correction coefficient, as
// the step evaluates them; the exact Hessian of each distance (the interior's by
// polarisation of its directional second derivative). H: the 6x6 over (p, a, b), upper
// triangle, kappa-scaled (no h^2). False when no term is active.
__device__ __noinline__ bool pair_block(const d2f_scene_desc &d, int ge, double2 xp, double2 xa, double2 xb, double *H) {
    const double dhat = d.ipc_dhat, kappa = d.ipc_kappa, dlo = 1.0e-9 * dhat;
    const double abx = xb.x - xa.x, aby = xb.y - xa.y;
    const double L2 = dmax(abx * abx + aby * aby, 1.0e-30), Ll = sqrt(L2);
    const double wx = xp.x - xa.x, wy = xp.y - xa.y;
    const double tt = (wx * abx + wy * aby) / L2;
    double dvx = wx - tt * abx, dvy = wy - tt * aby;
    if (tt <= 0.0) { dvx = wx; dvy = wy; }
    else if (tt >= 1.0) { dvx = xp.x - xb.x; dvy = xp.y - xb.y; }
    const double dd0 = sqrt(dvx * dvx + dvy * dvy);
    if (!(dd0 < d.reach)) return false;
    for (int q = 0; q < 21; ++q) H[q] = 0.0;
    bool any = false;
    if (tt > 0.0 && tt < 1.0 && dd0 < dhat) {
        const double dd = dmax(dd0, dlo), nx = dvx / dd, ny = dvy / dd;
        const double g[6] = {nx, ny, -(1.0 - tt) * nx, -(1.0 - tt) * ny, -tt * nx, -tt * ny};
        const double c0 = abx * wy - aby * wx;
        const double bp = barrier_bp<double>(dd, dhat), bpp = barrier_bpp<double>(dd, dhat);
        double q[6], v[6];
        for (int i = 0; i < 6; ++i) {
            for (int k = 0; k < 6; ++k) v[k] = k == i ? 1.0 : 0.0;
            q[i] = line_ddd(abx, aby, wx, wy, Ll, c0, v);
        }
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j) {
                double hd = q[i];
                if (j != i) {
                    for (int k = 0; k < 6; ++k) v[k] = (k == i || k == j) ? 1.0 : 0.0;
                    hd = 0.5 * (line_ddd(abx, aby, wx, wy, Ll, c0, v) - q[i] - q[j]);
                }
                H[ut6(i, j)] += kappa * (bpp * g[i] * g[j] + bp * hd);
            }
        any = true;
    }
    double coef_a = -d.ca[ge];
    if (tt <= 0.0) coef_a += 1.0;
    const double d_a = sqrt(wx * wx + wy * wy);
    if (coef_a != 0.0 && d_a < dhat) {
        point_block(coef_a, wx, wy, dmax(d_a, dlo), dhat, kappa, 1, H);
        any = true;
    }
    double coef_b = -d.cb[ge];
    if (tt >= 1.0) coef_b += 1.0;
    const double wbx = xp.x - xb.x, wby = xp.y - xb.y, d_b = sqrt(wbx * wbx + wby * wby);
    if (coef_b != 0.0 && d_b < dhat) {
        point_block(coef_b, wbx, wby, dmax(d_b, dlo), dhat, kappa, 2, H);
        any = true;
    }
    return any;
}

// ---- affine bodies (AffineBodies, implicit/affine.py:60-101, 156-269; the reference's
// adjoint refuses them): the system in the reduced coordinates, S^T H S + h^2 K_A with
// x = J q on a body's nodes (J = [w^T 0; 0 w^T], q = (t_x, A11, A12, t_y, A21, A22)) and K_A
// the body's exact elastic block at its A. Per body, QW doubles of the work buffer:
constexpr int QW = 112;
constexpr int Q_R = 0, Q_Z = 6, Q_P = 12, Q_AP = 18, Q_L = 24, Q_W = 30, Q_K = 36, Q_PI = 72;
// R, Z, P, AP, lam (6 each) of the CG; W = sum w w^T (00 01 02 11 12 22); K = h^2 K_A (6x6);
// PI = the inverse of the body's block preconditioner sum J^T diag(D) J + h^2 K_A (6x6).

// 3x3 symmetric solve by the adjugate (W from the node weights of one body: well conditioned)
__device__ __forceinline__ void sym3_solve(const double *W, const double *b, double *x) {
    const double a00 = W[0], a01 = W[1], a02 = W[2], a11 = W[3], a12 = W[4], a22 = W[5];
    const double c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22, c02 = a01 * a12 - a02 * a11;
    const double c11 = a00 * a22 - a02 * a02, c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
    const double det = a00 * c00 + a01 * c01 + a02 * c02, r = det != 0.0 ? 1.0 / det : 0.0;
    x[0] = (c00 * b[0] + c01 * b[1] + c02 * b[2]) * r;
    x[1] = (c01 * b[0] + c11 * b[1] + c12 * b[2]) * r;
    x[2] = (c02 * b[0] + c12 * b[1] + c22 * b[2]) * r;
}

// One body's setup from its node sums v (24: W = sum w w^T, sum D_x w w^T, sum D_y w w^T
// (6 each, 00 01 02 11 12 22), sum w x, sum w y (3 each)) and, warm, lw = sum w lam (6):
// W, h^2 K_A at the body's A, the inverse of its block preconditioner, lam_q and p_q. Out of
// line: its local 6x6 arrays would otherwise sit in every thread's frame of the CG kernel.
__device__ __noinline__ void affine_setup(double *qb, const double *v, const double *lw, int warm, double Mu,
                                          double La, double h2) {
    for (int q = 0; q < 6; ++q) qb[Q_W + q] = v[q];
    double qx[3], qy[3];
    sym3_solve(v, v + 18, qx);
    sym3_solve(v, v + 21, qy);
    const M2 A{qx[1], qx[2], qy[1], qy[2]};
    for (int q = 0; q < 36; ++q) qb[Q_K + q] = 0.0;
    const int idx[4] = {1, 2, 4, 5};
    for (int k = 0; k < 4; ++k) {
        const M2 E{k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0, k == 3 ? 1.0 : 0.0};
        const M2 col = nh_d2(A, E, Mu, La);
        const double cv[4] = {col.a, col.b, col.c, col.d};
        for (int r = 0; r < 4; ++r) qb[Q_K + 6 * idx[r] + idx[k]] = h2 * cv[r];
    }
    // the block preconditioner: Cholesky of the projected reduced Hessian, its inverse
    double H6[6][6], L6[6][6];
    reduced_hessian(A, Mu, La, h2, v + 6, H6);
    chol6(H6, L6);
    for (int c = 0; c < 6; ++c) {
        double e[6], xcol[6];
        for (int q = 0; q < 6; ++q) e[q] = q == c ? 1.0 : 0.0;
        chol6_solve(L6, e, xcol);
        for (int r = 0; r < 6; ++r) qb[Q_PI + 6 * r + c] = xcol[r];
    }
    double lx[3] = {0.0, 0.0, 0.0}, ly[3] = {0.0, 0.0, 0.0};
    if (warm) { sym3_solve(v, lw, lx); sym3_solve(v, lw + 3, ly); }
    for (int q = 0; q < 3; ++q) {
        qb[Q_L + q] = lx[q]; qb[Q_L + 3 + q] = ly[q];
        qb[Q_P + q] = lx[q]; qb[Q_P + 3 + q] = ly[q];
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) pcg_kernel(const __grid_constant__ d2f_scene_desc d, const double *__restrict__ xl,
                                                 const double *__restrict__ rhs, double *__restrict__ lam,
                                                 double *__restrict__ work, const double *__restrict__ tens, double rtol,
                                                 int max_iter, int warm, int *__restrict__ iters_out,
                                                 int *__restrict__ status_out) {
    constexpr int NW = NT / 32;
    __shared__ double red[NW * 4 + 4];
    __shared__ double s_col[MAXC][8];
    __shared__ int sc_next, s_stop, s_status, s_npair;
    __shared__ double s_alpha, s_beta, s_rz;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double h2 = d.dt * d.dt;
    const int N = d.N;
    const double2 *__restrict__ XL = reinterpret_cast<const double2 *>(xl);
    const double2 *__restrict__ B2 = reinterpret_cast<const double2 *>(rhs);
    double2 *__restrict__ LAM = reinterpret_cast<double2 *>(lam);
    double2 *__restrict__ R = reinterpret_cast<double2 *>(work);
    double2 *__restrict__ Z = R + N;
    double2 *__restrict__ P = R + 2 * N;
    double2 *__restrict__ AP = R + 3 * N;
    double2 *__restrict__ DI = R + 4 * N;
    double2 *__restrict__ EX = R + 5 * N;                       // P with the affine nodes' J p_q
    double *__restrict__ PB = work + 12 * (size_t)N;            // IPC pair blocks, 24 a candidate slot
    double *__restrict__ QB = PB + (d.Ne > 0 ? 24 * (size_t)d.cand_total : 0);   // affine bodies, QW each
    const double4_32a *__restrict__ Bm = reinterpret_cast<const double4_32a *>(d.Bm);
    const double *__restrict__ Ar = reinterpret_cast<const double *>(d.area);
    const double *__restrict__ Mu = reinterpret_cast<const double *>(d.mu);
    const double *__restrict__ La = reinterpret_cast<const double *>(d.lam);
    double4_32a *__restrict__ Esc = reinterpret_cast<double4_32a *>(d.escr);  // .x .y: K v per corner; .z .w: diagonal
    double *__restrict__ Ec = reinterpret_cast<double *>(d.ecache);          // F^-T, la log J - mu
    const double *__restrict__ TC = tens ? tens : d.t_Tcmd;
    if (tid < d.n_col && tid < MAXC)
        for (int q = 0; q < 8; ++q) s_col[tid][q] = d.colliders[8 * tid + q];

    for (;;) {
        if (tid == 0) sc_next = atomicAdd(d.work + 1, 1);
        block_barrier();
        const int sc = sc_next;
        if (sc >= d.n_scenes) break;
        const d2f_seg sg = d.segs[sc];
        const int n0 = sg.node0, n1 = sg.node0 + sg.nn, t0 = sg.tri0, t1 = sg.tri0 + sg.nt;
        const bool has_aff = sg.naff > 0, has_ipc = d.Ne > 0 && sg.ne > 0;
        // a DOF of the CG on the nodes: free and not slaved to an affine body
        auto plain = [&](int i, uint8_t fm, int c) -> bool { return (fm & (1 << c)) && d.node_aff[i] < 0; };
        auto J_of = [&](int i, double &w0, double &w1, double &w2) -> double * {
            const int ka = d.node_aff[i];
            const double *w = d.a_w + 3 * ka;
            w0 = w[0]; w1 = w[1]; w2 = w[2];
            return QB + (size_t)QW * d.a_grp[ka];
        };

        // AP = (M + h^2 (K_elastic + K_collider + K_tendon + K_spring + K_pressure + K_ipc)) V
        // for this scene, all DOFs
        auto hvp = [&](const double2 *__restrict__ V) {
            // element pass: corner shares of h^2 K_elastic V (hvp_elastic_kernel, implicit/adjoint.py:69-84)
            for (int t = t0 + tid; t < t1; t += NT) {
                const int i0 = d.tri[3 * t], i1 = d.tri[3 * t + 1], i2 = d.tri[3 * t + 2];
                const double *ec = Ec + 9 * (size_t)t;
                const double G00 = ec[0], G01 = ec[1], G10 = ec[2], G11 = ec[3], c1 = ec[4];
                const double2 p0 = V[i0], p1 = V[i1], p2 = V[i2];
                const double4_32a B = Bm[t];
                const double q1x = p1.x - p0.x, q1y = p1.y - p0.y, q2x = p2.x - p0.x, q2y = p2.y - p0.y;
                const double f00 = q1x * B.x + q2x * B.z, f01 = q1x * B.y + q2x * B.w;
                const double f10 = q1y * B.x + q2y * B.z, f11 = q1y * B.y + q2y * B.w;
                const double mu = Mu[t], la = La[t];
                const double GdF = G00 * f00 + G01 * f01 + G10 * f10 + G11 * f11;
                // d2Psi/dF2 [dF] = mu dF + la (G:dF) G - (la log J - mu) G dF^T G
                const double T00 = G00 * f00 + G01 * f01, T01 = G00 * f10 + G01 * f11;
                const double T10 = G10 * f00 + G11 * f01, T11 = G10 * f10 + G11 * f11;
                const double W00 = T00 * G00 + T01 * G10, W01 = T00 * G01 + T01 * G11;
                const double W10 = T10 * G00 + T11 * G10, W11 = T10 * G01 + T11 * G11;
                const double dP00 = mu * f00 + la * GdF * G00 - c1 * W00, dP01 = mu * f01 + la * GdF * G01 - c1 * W01;
                const double dP10 = mu * f10 + la * GdF * G10 - c1 * W10, dP11 = mu * f11 + la * GdF * G11 - c1 * W11;
                const double hA = h2 * Ar[t];
                const double h1x = hA * (dP00 * B.x + dP01 * B.y), h1y = hA * (dP10 * B.x + dP11 * B.y);
                const double h2x = hA * (dP00 * B.z + dP01 * B.w), h2y = hA * (dP10 * B.z + dP11 * B.w);
                double4_32a *e = Esc + 3 * t;
                e[0].x = -(h1x + h2x); e[0].y = -(h1y + h2y);
                e[1].x = h1x; e[1].y = h1y;
                e[2].x = h2x; e[2].y = h2y;
            }
            block_barrier();
            // node pass: inertia + gathered corners (ascending triangle) + frozen collider barrier
            for (int i = n0 + tid; i < n1; i += NT) {
                const double2 pi = V[i];
                const double m = d.mass[i];
                double ax = m * pi.x, ay = m * pi.y;
                for (int k = d.inc_ptr[i]; k < d.inc_ptr[i + 1]; ++k) {
                    const double4_32a c = Esc[d.inc[k]];
                    ax += c.x; ay += c.y;
                }
                if (d.node_bslot[i] >= 0) {
                    const double2 xi = XL[i];
                    for (int k = 0; k < d.n_col; ++k) {
                        double h00, h01, h11;
                        collider_hessian(s_col[k], (int)s_col[k][0], xi.x, xi.y, d.dhat, d.kappa, h00, h01, h11);
                        ax += h2 * (h00 * pi.x + h01 * pi.y);
                        ay += h2 * (h01 * pi.x + h11 * pi.y);
                    }
                }
                AP[i] = make_double2(ax, ay);
            }
            block_barrier();
            if (sg.nten > 0) {
                // tendon (tension-controlled): geometric stiffness T/len (I - d d^T) per segment,
                // the term of pHp_tendon_kernel (implicit/actuation.py:229-248)
                for (int j = sg.tent0 + tid; j < sg.tent0 + sg.ntent; j += NT) {
                    const int n = d.t_node[j], k = d.t_tid[j];
                    const double tau = dmax(TC[k], 0.0);
                    double ax = 0.0, ay = 0.0;
                    const double2 xn = XL[n], pn = V[n];
                    const int nb[2] = {d.t_prv[j], d.t_nxt[j]};
                    for (int s2 = 0; s2 < 2; ++s2) {
                        if (nb[s2] < 0) continue;
                        const int o = d.t_node[nb[s2]];
                        const double2 xo = XL[o], po = V[o];
                        const double tx = xn.x - xo.x, ty = xn.y - xo.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                        const double sx = tx / ln, sy = ty / ln;
                        const double dx = pn.x - po.x, dy = pn.y - po.y, al = dx * sx + dy * sy;
                        ax += tau / ln * (dx - al * sx);
                        ay += tau / ln * (dy - al * sy);
                    }
                    atomicAdd(&AP[n].x, h2 * ax);
                    atomicAdd(&AP[n].y, h2 * ay);
                }
                block_barrier();
            }
            if (sg.nsp > 0 || sg.npe > 0) {
                // springs: h^2 (k n n^T + k (1 - L0/|d|) (I - n n^T)) on the ends' difference
                // (Springs, implicit/actuation.py:381-393), the tangential term unclamped (the
                // exact tangent)
                for (int k = sg.sp0 + tid; k < sg.sp0 + sg.nsp; k += NT) {
                    const int a = d.sp_a[k], b = d.sp_b[k];
                    const double2 xa = XL[a], xb = b >= 0 ? XL[b] : make_double2(d.sp_anchor[2 * k], d.sp_anchor[2 * k + 1]);
                    const double dx = xa.x - xb.x, dy = xa.y - xb.y, ln = sqrt(dx * dx + dy * dy + 1.0e-30);
                    const double nx = dx / ln, ny = dy / ln, kk = d.sp_k[k], kt = kk * (1.0 - d.sp_L0[k] / ln);
                    double vx = V[a].x, vy = V[a].y;
                    if (b >= 0) { vx -= V[b].x; vy -= V[b].y; }
                    const double al = vx * nx + vy * ny;
                    const double fx = h2 * (kk * al * nx + kt * (vx - al * nx)), fy = h2 * (kk * al * ny + kt * (vy - al * ny));
                    atomicAdd(&AP[a].x, fx); atomicAdd(&AP[a].y, fy);
                    if (b >= 0) { atomicAdd(&AP[b].x, -fx); atomicAdd(&AP[b].y, -fy); }
                }
                // pressure: the gradient -h^2 p/2 (t.y, -t.x) on both ends of an edge is linear in
                // x, so its product with V is the same with t -> V_b - V_a (Pressure, :98-118)
                for (int e = sg.pe0 + tid; e < sg.pe0 + sg.npe; e += NT) {
                    const int a = d.pe_a[e], b = d.pe_b[e];
                    const double sp = -0.5 * h2 * d.ch_p[d.pe_ch[e]];
                    const double tx = V[b].x - V[a].x, ty = V[b].y - V[a].y;
                    atomicAdd(&AP[a].x, sp * ty); atomicAdd(&AP[a].y, -sp * tx);
                    atomicAdd(&AP[b].x, sp * ty); atomicAdd(&AP[b].y, -sp * tx);
                }
                block_barrier();
            }
            if (has_ipc) {  // the frozen pair blocks, h^2 H_pair V
                const int np = s_npair < sg.ncap ? s_npair : sg.ncap;
                for (int c = tid; c < np; c += NT) {
                    const double *pb = PB + 24 * (size_t)(sg.cand0 + c);
                    const int ids[3] = {(int)pb[21], (int)pb[22], (int)pb[23]};
                    double v[6], o[6];
                    for (int q = 0; q < 3; ++q) { v[2 * q] = V[ids[q]].x; v[2 * q + 1] = V[ids[q]].y; }
                    for (int r = 0; r < 6; ++r) {
                        double acc = 0.0;
                        for (int q = 0; q < 6; ++q) acc += pb[r <= q ? ut6(r, q) : ut6(q, r)] * v[q];
                        o[r] = h2 * acc;
                    }
                    for (int q = 0; q < 3; ++q) { atomicAdd(&AP[ids[q]].x, o[2 * q]); atomicAdd(&AP[ids[q]].y, o[2 * q + 1]); }
                }
                block_barrier();
            }
        };
        // the affine bodies' share of a product: AP_q = sum J^T AP (a warp per body, fixed
        // shuffle tree) + h^2 K_A p_q
        auto gather_q = [&]() {
            for (int b = sg.aff0 + warp; b < sg.aff0 + sg.naff; b += NW) {
                double *qb = QB + (size_t)QW * b;
                double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                for (int k = d.a_ptr[b] + lane; k < d.a_ptr[b + 1]; k += 32) {
                    const int i = d.a_node[k];
                    const double *w = d.a_w + 3 * k;
                    const double2 a = AP[i];
                    v[0] += w[0] * a.x; v[1] += w[1] * a.x; v[2] += w[2] * a.x;
                    v[3] += w[0] * a.y; v[4] += w[1] * a.y; v[5] += w[2] * a.y;
                }
                for (int q = 0; q < 6; ++q) v[q] = wsum_all(v[q]);  // lanes 0-5 each write one
                if (lane < 6) {
                    double kp = 0.0;
                    for (int q = 0; q < 6; ++q) kp += qb[Q_K + 6 * lane + q] * qb[Q_P + q];
                    double vv = v[0];
                    for (int q = 1; q < 6; ++q) if (lane == q) vv = v[q];
                    qb[Q_AP + lane] = vv + kp;
                }
            }
            block_barrier();
        };
        // EX = P on the plain nodes, J p_q on the affine ones
        auto expand = [&](const double2 *__restrict__ V, int qoff) {
            for (int i = n0 + tid; i < n1; i += NT) {
                if (d.node_aff[i] < 0) { EX[i] = V[i]; continue; }
                double w0, w1, w2;
                const double *qb = J_of(i, w0, w1, w2);
                const double *q = qb + qoff;
                EX[i] = make_double2(w0 * q[0] + w1 * q[1] + w2 * q[2], w0 * q[3] + w1 * q[4] + w2 * q[5]);
            }
            block_barrier();
        };

        // ---- tangent at x_lin: F^-T and (la log J - mu) per triangle, the Jacobi diagonal per corner
        for (int t = t0 + tid; t < t1; t += NT) {
            const int i0 = d.tri[3 * t], i1 = d.tri[3 * t + 1], i2 = d.tri[3 * t + 2];
            const double2 x0 = XL[i0], x1 = XL[i1], x2 = XL[i2];
            const double4_32a B = Bm[t];
            const double e1x = x1.x - x0.x, e1y = x1.y - x0.y, e2x = x2.x - x0.x, e2y = x2.y - x0.y;
            const double F00 = e1x * B.x + e2x * B.z, F01 = e1x * B.y + e2x * B.w;
            const double F10 = e1y * B.x + e2y * B.z, F11 = e1y * B.y + e2y * B.w;
            const double J = F00 * F11 - F10 * F01, logJ = log(dmax(J, 1.0e-6));
            const double iJ = J != 0.0 ? 1.0 / J : 0.0;
            const double G00 = F11 * iJ, G01 = -F10 * iJ, G10 = -F01 * iJ, G11 = F00 * iJ;
            const double mu = Mu[t], la = La[t], c1 = la * logJ - mu, kk = la - c1, hA = h2 * Ar[t];
            double *ec = Ec + 9 * (size_t)t;
            ec[0] = G00; ec[1] = G01; ec[2] = G10; ec[3] = G11; ec[4] = c1;
            const double bx[3] = {-(B.x + B.z), B.x, B.z}, by[3] = {-(B.y + B.w), B.y, B.w};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double bb = mu * (bx[c] * bx[c] + by[c] * by[c]);
                const double gx = G00 * bx[c] + G01 * by[c], gy = G10 * bx[c] + G11 * by[c];
                Esc[3 * t + c] = make_double4_32a(0.0, 0.0, hA * dmax(bb + kk * gx * gx, 0.0), hA * dmax(bb + kk * gy * gy, 0.0));
            }
        }
        if (tid == 0) { s_stop = 0; s_status = 0; s_npair = 0; }
        block_barrier();
        // ---- the frozen IPC pair blocks at x_lin: every node-edge pair of the scene tested
        if (has_ipc) {
            const int nbs = sg.nb;
            const long npairs = (long)sg.ne * nbs;
            for (long c = tid; c < npairs; c += NT) {
                const int k = (int)(c / nbs), j = (int)(c % nbs);
                const int ge = sg.edge0 + k, a = d.ea[ge], b = d.eb[ge], pn = d.bnd[sg.bnd0 + j];
                if (pn == a || pn == b) continue;
                if (excluded(d, sg.bnd0 + j, d.ela[ge]) || excluded(d, sg.bnd0 + j, d.elb[ge])) continue;
                double H[21];
                if (!pair_block(d, ge, XL[pn], XL[a], XL[b], H)) continue;
                const int slot = atomicAdd(&s_npair, 1);
                if (slot >= sg.ncap) continue;
                double *pb = PB + 24 * (size_t)(sg.cand0 + slot);
                for (int q = 0; q < 21; ++q) pb[q] = H[q];
                pb[21] = pn; pb[22] = a; pb[23] = b;
            }
            block_barrier();
            if (tid == 0 && s_npair > sg.ncap) { s_stop = 1; s_status = D2F_ECAP; }
        }
        // ---- the Jacobi preconditioner; the initial guess (0, or lam as given with warm)
        for (int i = n0 + tid; i < n1; i += NT) {
            const double m = d.mass[i];
            double dx = m, dy = m;
            for (int k = d.inc_ptr[i]; k < d.inc_ptr[i + 1]; ++k) {
                const double4_32a c = Esc[d.inc[k]];
                dx += c.z; dy += c.w;
            }
            if (d.node_bslot[i] >= 0) {
                const double2 xi = XL[i];
                for (int k = 0; k < d.n_col; ++k) {
                    double h00, h01, h11;
                    collider_hessian(s_col[k], (int)s_col[k][0], xi.x, xi.y, d.dhat, d.kappa, h00, h01, h11);
                    dx += h2 * dmax(h00, 0.0); dy += h2 * dmax(h11, 0.0);
                }
            }
            DI[i] = make_double2(dx, dy);
        }
        block_barrier();
        for (int k = sg.sp0 + tid; k < sg.sp0 + sg.nsp; k += NT) {  // springs' diagonal (clamped, as the step's)
            const int a = d.sp_a[k], b = d.sp_b[k];
            const double2 xa = XL[a], xb = b >= 0 ? XL[b] : make_double2(d.sp_anchor[2 * k], d.sp_anchor[2 * k + 1]);
            const double dx = xa.x - xb.x, dy = xa.y - xb.y, ln = sqrt(dx * dx + dy * dy + 1.0e-30);
            const double nx = dx / ln, ny = dy / ln, kk = d.sp_k[k], kt = dmax(kk * (1.0 - d.sp_L0[k] / ln), 0.0);
            const double hx = h2 * (kk * nx * nx + kt * (1.0 - nx * nx)), hy = h2 * (kk * ny * ny + kt * (1.0 - ny * ny));
            atomicAdd(&DI[a].x, hx); atomicAdd(&DI[a].y, hy);
            if (b >= 0) { atomicAdd(&DI[b].x, hx); atomicAdd(&DI[b].y, hy); }
        }
        if (has_ipc) {  // the pair blocks' diagonals, clamped
            const int np = s_npair < sg.ncap ? s_npair : sg.ncap;
            for (int c = tid; c < np; c += NT) {
                const double *pb = PB + 24 * (size_t)(sg.cand0 + c);
                for (int q = 0; q < 3; ++q) {
                    const int n = (int)pb[21 + q];
                    atomicAdd(&DI[n].x, h2 * dmax(pb[ut6(2 * q, 2 * q)], 0.0));
                    atomicAdd(&DI[n].y, h2 * dmax(pb[ut6(2 * q + 1, 2 * q + 1)], 0.0));
                }
            }
        }
        block_barrier();
        if (has_aff) {
            // per body: its A from x_lin (least squares over its nodes: x = J q holds there), the
            // exact block h^2 K_A, and the inverse of the block preconditioner sum J^T D J +
            // h^2 K_A (the forward's reduced Hessian, projected SPD, by Cholesky); the initial
            // lam_q from lam on its nodes (warm) or 0
            for (int b = sg.aff0 + warp; b < sg.aff0 + sg.naff; b += NW) {
                double v[24];
                for (int q = 0; q < 24; ++q) v[q] = 0.0;
                for (int k = d.a_ptr[b] + lane; k < d.a_ptr[b + 1]; k += 32) {
                    const int i = d.a_node[k];
                    const double *w = d.a_w + 3 * k;
                    const double2 x = XL[i], dg = DI[i];
                    const double o[6] = {w[0] * w[0], w[0] * w[1], w[0] * w[2], w[1] * w[1], w[1] * w[2], w[2] * w[2]};
                    for (int q = 0; q < 6; ++q) { v[q] += o[q]; v[6 + q] += dg.x * o[q]; v[12 + q] += dg.y * o[q]; }
                    for (int q = 0; q < 3; ++q) { v[18 + q] += w[q] * x.x; v[21 + q] += w[q] * x.y; }
                }
                for (int q = 0; q < 24; ++q) v[q] = wsum(v[q]);
                double lw[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                if (warm) {
                    for (int k = d.a_ptr[b] + lane; k < d.a_ptr[b + 1]; k += 32) {
                        const double *w = d.a_w + 3 * k;
                        const double2 l = LAM[d.a_node[k]];
                        for (int q = 0; q < 3; ++q) { lw[q] += w[q] * l.x; lw[3 + q] += w[q] * l.y; }
                    }
                    for (int q = 0; q < 6; ++q) lw[q] = wsum(lw[q]);
                }
                if (lane == 0) affine_setup(QB + (size_t)QW * b, v, lw, warm, d.a_Mu[b], d.a_La[b], h2);
                __syncwarp();
            }
            block_barrier();
        }
        for (int i = n0 + tid; i < n1; i += NT) {
            const uint8_t fm = d.free_mask[i];
            const double2 dd = DI[i];
            DI[i] = make_double2(plain(i, fm, 0) ? 1.0 / dd.x : 0.0, plain(i, fm, 1) ? 1.0 / dd.y : 0.0);
            double2 l0 = make_double2(0.0, 0.0);
            if (warm) {
                const double2 l = LAM[i];
                l0 = make_double2(plain(i, fm, 0) ? l.x : 0.0, plain(i, fm, 1) ? l.y : 0.0);
            }
            LAM[i] = l0;
            P[i] = l0;
        }
        block_barrier();
        if (warm) {  // A lam0
            if (has_aff) expand(P, Q_P);
            hvp(has_aff ? EX : P);
            if (has_aff) gather_q();
        }
        // r = b - A lam0 on the plain DOFs and the bodies' coordinates, z = D^-1 r, p = z
        double acc[3] = {0.0, 0.0, 0.0};
        for (int i = n0 + tid; i < n1; i += NT) {
            const uint8_t fm = d.free_mask[i];
            const double2 b = B2[i], di = DI[i];
            const double2 a = warm ? AP[i] : make_double2(0.0, 0.0);
            const double rx = plain(i, fm, 0) ? b.x - a.x : 0.0, ry = plain(i, fm, 1) ? b.y - a.y : 0.0;
            R[i] = make_double2(rx, ry);
            const double zx = di.x * rx, zy = di.y * ry;
            Z[i] = make_double2(zx, zy);
            P[i] = make_double2(zx, zy);
            acc[0] += rx * zx + ry * zy;
            acc[1] += rx * rx + ry * ry;
            acc[2] += (plain(i, fm, 0) ? b.x * b.x : 0.0) + (plain(i, fm, 1) ? b.y * b.y : 0.0);
        }
        if (has_aff) {
            // b_q = sum J^T b (a warp per body), r_q = b_q - A_q lam0, then z_q = PI r_q, p_q = z_q
            for (int b = sg.aff0 + warp; b < sg.aff0 + sg.naff; b += NW) {
                double *qb = QB + (size_t)QW * b;
                double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                for (int k = d.a_ptr[b] + lane; k < d.a_ptr[b + 1]; k += 32) {
                    const double *w = d.a_w + 3 * k;
                    const double2 bb = B2[d.a_node[k]];
                    v[0] += w[0] * bb.x; v[1] += w[1] * bb.x; v[2] += w[2] * bb.x;
                    v[3] += w[0] * bb.y; v[4] += w[1] * bb.y; v[5] += w[2] * bb.y;
                }
                for (int q = 0; q < 6; ++q) v[q] = wsum(v[q]);
                if (lane == 0)
                    for (int q = 0; q < 6; ++q) {
                        qb[Q_R + q] = v[q] - (warm ? qb[Q_AP + q] : 0.0);
                        acc[2] += v[q] * v[q];
                    }
            }
            block_barrier();
            for (int b = sg.aff0 + warp; b < sg.aff0 + sg.naff; b += NW) {
                double *qb = QB + (size_t)QW * b;
                if (lane < 6) {
                    double z = 0.0;
                    for (int q = 0; q < 6; ++q) z += qb[Q_PI + 6 * lane + q] * qb[Q_R + q];
                    qb[Q_Z + lane] = z;
                    qb[Q_P + lane] = z;
                }
                __syncwarp();
                if (lane == 0)
                    for (int q = 0; q < 6; ++q) { acc[0] += qb[Q_R + q] * qb[Q_Z + q]; acc[1] += qb[Q_R + q] * qb[Q_R + q]; }
            }
        }
        bsum<NT, 3>(acc, red);
        const double bb = acc[2];
        if (tid == 0) s_rz = acc[0];
        block_barrier();
        int it = 0;
        double rr = acc[1];
        for (; it < max_iter; ++it) {
            if (!(rr > rtol * rtol * bb) || s_stop) break;
            if (has_aff) expand(P, Q_P);
            hvp(has_aff ? EX : P);
            if (has_aff) gather_q();
            // ---- alpha = rz / p.Ap
            double pa[1] = {0.0};
            for (int i = n0 + tid; i < n1; i += NT) {
                const uint8_t fm = d.free_mask[i];
                const double2 pi = P[i], ai = AP[i];
                pa[0] += (plain(i, fm, 0) ? pi.x * ai.x : 0.0) + (plain(i, fm, 1) ? pi.y * ai.y : 0.0);
            }
            for (int b = sg.aff0 + warp; has_aff && b < sg.aff0 + sg.naff; b += NW)
                if (lane == 0) {
                    const double *qb = QB + (size_t)QW * b;
                    for (int q = 0; q < 6; ++q) pa[0] += qb[Q_P + q] * qb[Q_AP + q];
                }
            bsum<NT, 1>(pa, red);
            if (tid == 0) {
                if (!(pa[0] > 0.0)) { s_stop = 1; s_status = D2F_ENAN; }  // not positive definite along p
                s_alpha = pa[0] > 0.0 ? s_rz / pa[0] : 0.0;
            }
            block_barrier();
            if (s_stop) break;
            const double al = s_alpha;
            double nr[2] = {0.0, 0.0};
            for (int i = n0 + tid; i < n1; i += NT) {
                const uint8_t fm = d.free_mask[i];
                const double2 pi = P[i], ai = AP[i], li = LAM[i], ri = R[i], di = DI[i];
                LAM[i] = make_double2(li.x + al * pi.x, li.y + al * pi.y);
                const double rx = plain(i, fm, 0) ? ri.x - al * ai.x : 0.0, ry = plain(i, fm, 1) ? ri.y - al * ai.y : 0.0;
                R[i] = make_double2(rx, ry);
                const double zx = di.x * rx, zy = di.y * ry;
                Z[i] = make_double2(zx, zy);
                nr[0] += rx * zx + ry * zy;
                nr[1] += rx * rx + ry * ry;
            }
            if (has_aff) {
                for (int b = sg.aff0 + warp; b < sg.aff0 + sg.naff; b += NW) {
                    double *qb = QB + (size_t)QW * b;
                    if (lane < 6) {
                        qb[Q_L + lane] += al * qb[Q_P + lane];
                        qb[Q_R + lane] -= al * qb[Q_AP + lane];
                    }
                    __syncwarp();
                    if (lane < 6) {
                        double z = 0.0;
                        for (int q = 0; q < 6; ++q) z += qb[Q_PI + 6 * lane + q] * qb[Q_R + q];
                        qb[Q_Z + lane] = z;
                    }
                    __syncwarp();
                    if (lane == 0)
                        for (int q = 0; q < 6; ++q) { nr[0] += qb[Q_R + q] * qb[Q_Z + q]; nr[1] += qb[Q_R + q] * qb[Q_R + q]; }
                }
            }
            bsum<NT, 2>(nr, red);
            rr = nr[1];
            if (tid == 0) { s_beta = nr[0] / s_rz; s_rz = nr[0]; }
            block_barrier();
            const double be = s_beta;
            for (int i = n0 + tid; i < n1; i += NT) {
                const double2 zi = Z[i], pi = P[i];
                P[i] = make_double2(zi.x + be * pi.x, zi.y + be * pi.y);
            }
            for (int b = sg.aff0 + warp; has_aff && b < sg.aff0 + sg.naff; b += NW) {
                double *qb = QB + (size_t)QW * b;
                if (lane < 6) qb[Q_P + lane] = qb[Q_Z + lane] + be * qb[Q_P + lane];
            }
            block_barrier();
        }
        if (has_aff) {  // lam on the bodies' nodes: J lam_q
            expand(LAM, Q_L);
            for (int i = n0 + tid; i < n1; i += NT)
                if (d.node_aff[i] >= 0) LAM[i] = EX[i];
            block_barrier();
        }
        if (tid == 0) {
            iters_out[sc] = it;
            status_out[sc] = s_status ? s_status : (rr > rtol * rtol * bb ? 1 : 0);
        }
        block_barrier();
    }
}

// dL/ds_e (s_e a scale on the element's mu and lambda) += -h^2 lam . f_e(x): the explicit
// dependence of the step residual on the element stiffness (drho_kernel, implicit/adjoint.py:164-178)
__global__ void vjp_scale_kernel(const __grid_constant__ d2f_scene_desc d, const double *__restrict__ xl,
                                 const double *__restrict__ lam, double *__restrict__ dscale) {
    const double h2 = d.dt * d.dt;
    const double2 *XL = reinterpret_cast<const double2 *>(xl);
    const double2 *LM = reinterpret_cast<const double2 *>(lam);
    const double4_32a *Bm = reinterpret_cast<const double4_32a *>(d.Bm);
    const double *Ar = reinterpret_cast<const double *>(d.area);
    const double *Mu = reinterpret_cast<const double *>(d.mu);
    const double *La = reinterpret_cast<const double *>(d.lam);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < d.T; t += gridDim.x * blockDim.x) {
        const int i0 = d.tri[3 * t], i1 = d.tri[3 * t + 1], i2 = d.tri[3 * t + 2];
        const double2 x0 = XL[i0], x1 = XL[i1], x2 = XL[i2];
        const double4_32a B = Bm[t];
        const double e1x = x1.x - x0.x, e1y = x1.y - x0.y, e2x = x2.x - x0.x, e2y = x2.y - x0.y;
        const M2 F{e1x * B.x + e2x * B.z, e1x * B.y + e2x * B.w, e1y * B.x + e2y * B.z, e1y * B.y + e2y * B.w};
        const M2 P = nh_P(F, Mu[t], La[t]);
        const double A = Ar[t];
        const double g1x = A * (P.a * B.x + P.b * B.y), g1y = A * (P.c * B.x + P.d * B.y);
        const double g2x = A * (P.a * B.z + P.b * B.w), g2y = A * (P.c * B.z + P.d * B.w);
        const double2 l0 = LM[i0], l1 = LM[i1], l2 = LM[i2];
        const double s = l0.x * (-(g1x + g2x)) + l0.y * (-(g1y + g2y)) + l1.x * g1x + l1.y * g1y + l2.x * g2x + l2.y * g2y;
        dscale[t] += -h2 * s;
    }
}

// dL/dp (gauge pressure of each chamber at this step) = -lam . dg/dp with the pressure
// gradient g_a = g_b = -h^2 p / 2 (t.y, -t.x), t = x_b - x_a, per edge (grad_pressure_kernel,
// implicit/actuation.py:98-108): + h^2 / 2 (lam_a + lam_b) . (t.y, -t.x), one thread per edge
__global__ void vjp_pressure_kernel(const __grid_constant__ d2f_scene_desc d, const double *__restrict__ xl,
                                    const double *__restrict__ lam, double *__restrict__ dp) {
    const double2 *X = reinterpret_cast<const double2 *>(xl);
    const double2 *L = reinterpret_cast<const double2 *>(lam);
    const double h2 = d.dt * d.dt;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d.n_pe; e += gridDim.x * blockDim.x) {
        const int a = d.pe_a[e], b = d.pe_b[e];
        const double tx = X[b].x - X[a].x, ty = X[b].y - X[a].y;
        const double lx = L[a].x + L[b].x, ly = L[a].y + L[b].y;
        atomicAdd(dp + d.pe_ch[e], 0.5 * h2 * (lx * ty - ly * tx));
    }
}

// dL/dT (tension of each tendon at this step) = -h^2 lam . dlen/dx: one block per scene, one
// thread per tendon of the scene, summed over its eyelets in eyelet order (deterministic)
__global__ void vjp_tension_kernel(const __grid_constant__ d2f_scene_desc d, const double *__restrict__ xl,
                                   const double *__restrict__ lam, double *__restrict__ dtension) {
    const double h2 = d.dt * d.dt;
    const double2 *XL = reinterpret_cast<const double2 *>(xl);
    const double2 *LM = reinterpret_cast<const double2 *>(lam);
    for (int sc = blockIdx.x; sc < d.n_scenes; sc += gridDim.x) {
        const d2f_seg sg = d.segs[sc];
        for (int k = sg.ten0 + threadIdx.x; k < sg.ten0 + sg.nten; k += blockDim.x) {
            double s = 0.0;
            for (int j = sg.tent0; j < sg.tent0 + sg.ntent; ++j) {
                if (d.t_tid[j] != k) continue;
                const int n = d.t_node[j];
                const double2 xn = XL[n], ln_ = LM[n];
                double gx = 0.0, gy = 0.0;
                if (d.t_prv[j] >= 0) {
                    const double2 xa = XL[d.t_node[d.t_prv[j]]];
                    const double tx = xn.x - xa.x, ty = xn.y - xa.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                    gx += tx / ln; gy += ty / ln;
                }
                if (d.t_nxt[j] >= 0) {
                    const double2 xb = XL[d.t_node[d.t_nxt[j]]];
                    const double tx = xb.x - xn.x, ty = xb.y - xn.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                    gx -= tx / ln; gy -= ty / ln;
                }
                s += ln_.x * gx + ln_.y * gy;
            }
            dtension[k] = -h2 * s;
        }
    }
}

}  // namespace adj
}  // namespace d2f

extern "C" {

int64_t d2f_adjoint_work_doubles(const d2f_solver *s) {
    if (!s) return 0;
    return 12 * (int64_t)s->d.N + (s->d.Ne > 0 ? 24 * (int64_t)s->d.cand_total : 0) +
           (int64_t)d2f::adj::QW * s->d.n_aff;
}

int32_t d2f_adjoint_solve(d2f_solver *s, const double *x_lin, const double *rhs, double *lam, double *work,
                          const double *tension, double rtol, int32_t max_iter, int32_t warm_start, int32_t *iters,
                          int32_t *status, void *stream) {
    g_err[0] = 0;
    if (!s || !x_lin || !rhs || !lam || !work || !iters || !status)
        return d2f_fail(D2F_EINVAL, "d2f_adjoint_solve: null argument");
    if (s->d.precision != D2F_FP64) return d2f_fail(D2F_EINVAL, "d2f_adjoint_solve: needs an FP64 solver");
    if (!(rtol > 0.0) || max_iter <= 0) return d2f_fail(D2F_EINVAL, "d2f_adjoint_solve: rtol > 0 and max_iter > 0");
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(s->d.work, 0, 4 * sizeof(int32_t), st) != cudaSuccess)
        return d2f_fail(D2F_ECUDA, "d2f_adjoint_solve: cudaMemsetAsync failed");
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return d2f_fail(D2F_ECUDA, "d2f_adjoint_solve: no CUDA device");
    // few scenes: 256 threads a scene, one block per SM at most; else 128 threads, 4 per SM
    const bool wide = d2f_default_threads(s->d) >= 256;
    int grid = nsm * (wide ? 1 : 4);
    if (grid > s->d.n_scenes) grid = s->d.n_scenes;
    if (wide)
        d2f::adj::pcg_kernel<256><<<grid, 256, 0, st>>>(s->d, x_lin, rhs, lam, work, tension, rtol, max_iter,
                                                       warm_start ? 1 : 0, iters, status);
    else
        d2f::adj::pcg_kernel<128><<<grid, 128, 0, st>>>(s->d, x_lin, rhs, lam, work, tension, rtol, max_iter,
                                                       warm_start ? 1 : 0, iters, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "d2f_adjoint_solve: launch failed: %s", cudaGetErrorString(e));
        return D2F_ECUDA;
    }
    return D2F_OK;
}

int32_t d2f_adjoint_vjp(d2f_solver *s, const double *x_lin, const double *lam, double *dscale, double *dtension,
                        void *stream) {
    g_err[0] = 0;
    if (!s || !x_lin || !lam || !dscale) return d2f_fail(D2F_EINVAL, "d2f_adjoint_vjp: null argument");
    if (s->d.precision != D2F_FP64) return d2f_fail(D2F_EINVAL, "d2f_adjoint_vjp: needs an FP64 solver");
    cudaStream_t st = (cudaStream_t)stream;
    d2f::adj::vjp_scale_kernel<<<(s->d.T + 255) / 256, 256, 0, st>>>(s->d, x_lin, lam, dscale);
    if (dtension && s->d.n_ten > 0)
        d2f::adj::vjp_tension_kernel<<<s->d.n_scenes < 4096 ? s->d.n_scenes : 4096, 32, 0, st>>>(s->d, x_lin, lam,
                                                                                              dtension);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "d2f_adjoint_vjp: launch failed: %s", cudaGetErrorString(e));
        return D2F_ECUDA;
    }
    return D2F_OK;
}

int32_t d2f_adjoint_vjp_pressure(d2f_solver *s, const double *x_lin, const double *lam, double *dpressure,
                                 void *stream) {
    g_err[0] = 0;
    if (!s || !x_lin || !lam || !dpressure) return d2f_fail(D2F_EINVAL, "d2f_adjoint_vjp_pressure: null argument");
    if (s->d.precision != D2F_FP64) return d2f_fail(D2F_EINVAL, "d2f_adjoint_vjp_pressure: needs an FP64 solver");
    if (s->d.n_pe <= 0) return D2F_OK;
    const int blocks = (s->d.n_pe + 255) / 256 < 1024 ? (s->d.n_pe + 255) / 256 : 1024;
    d2f::adj::vjp_pressure_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(s->d, x_lin, lam, dpressure);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "d2f_adjoint_vjp_pressure: launch failed: %s", cudaGetErrorString(e));
        return D2F_ECUDA;
    }
    return D2F_OK;
}

}  // extern "C"
