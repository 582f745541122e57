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

namespace d2f {
namespace adj {

constexpr int MAXC = 16;

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
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

template <int NT>
__global__ void __launch_bounds__(NT) pcg_kernel(const __grid_constant__ d2f_scene_desc d, const double *__restrict__ xl,
                                                 const double *__restrict__ rhs, double *__restrict__ lam,
                                                 double *__restrict__ work, const double *__restrict__ tens, double rtol,
                                                 int max_iter, int warm, int *__restrict__ iters_out,
                                                 int *__restrict__ status_out) {
    constexpr int NW = NT / 32;
    __shared__ double red[NW * 4 + 4];
    __shared__ double s_col[MAXC][8];
    __shared__ int sc_next, s_stop, s_status;
    __shared__ double s_alpha, s_beta, s_rz;
    const int tid = threadIdx.x;
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

        // AP = (M + h^2 (K_elastic + K_collider + K_tendon)) V for this scene, all DOFs
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
        if (tid == 0) { s_stop = 0; s_status = 0; }
        block_barrier();
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
        block_barrier();
        for (int i = n0 + tid; i < n1; i += NT) {
            const uint8_t fm = d.free_mask[i];
            const double2 dd = DI[i];
            DI[i] = make_double2((fm & 1) ? 1.0 / dd.x : 0.0, (fm & 2) ? 1.0 / dd.y : 0.0);
            double2 l0 = make_double2(0.0, 0.0);
            if (warm) {
                const double2 l = LAM[i];
                l0 = make_double2((fm & 1) ? l.x : 0.0, (fm & 2) ? l.y : 0.0);
            }
            LAM[i] = l0;
            P[i] = l0;
        }
        block_barrier();
        if (warm) hvp(P);  // A lam0
        // r = b - A lam0 on the free DOFs, z = D^-1 r, p = z
        double acc[3] = {0.0, 0.0, 0.0};
        for (int i = n0 + tid; i < n1; i += NT) {
            const uint8_t fm = d.free_mask[i];
            const double2 b = B2[i], di = DI[i];
            const double2 a = warm ? AP[i] : make_double2(0.0, 0.0);
            const double rx = (fm & 1) ? b.x - a.x : 0.0, ry = (fm & 2) ? b.y - a.y : 0.0;
            R[i] = make_double2(rx, ry);
            const double zx = di.x * rx, zy = di.y * ry;
            Z[i] = make_double2(zx, zy);
            P[i] = make_double2(zx, zy);
            acc[0] += rx * zx + ry * zy;
            acc[1] += rx * rx + ry * ry;
            acc[2] += ((fm & 1) ? b.x * b.x : 0.0) + ((fm & 2) ? b.y * b.y : 0.0);
        }
        bsum<NT, 3>(acc, red);
        const double bb = acc[2];
        if (tid == 0) s_rz = acc[0];
        block_barrier();
        int it = 0;
        double rr = acc[1];
        for (; it < max_iter; ++it) {
            if (!(rr > rtol * rtol * bb) || s_stop) break;
            hvp(P);
            // ---- alpha = rz / p.Ap
            double pa[1] = {0.0};
            for (int i = n0 + tid; i < n1; i += NT) {
                const uint8_t fm = d.free_mask[i];
                const double2 pi = P[i], ai = AP[i];
                pa[0] += ((fm & 1) ? pi.x * ai.x : 0.0) + ((fm & 2) ? pi.y * ai.y : 0.0);
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
                const double rx = (fm & 1) ? ri.x - al * ai.x : 0.0, ry = (fm & 2) ? ri.y - al * ai.y : 0.0;
                R[i] = make_double2(rx, ry);
                const double zx = di.x * rx, zy = di.y * ry;
                Z[i] = make_double2(zx, zy);
                nr[0] += rx * zx + ry * zy;
                nr[1] += rx * rx + ry * ry;
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

int32_t d2f_adjoint_solve(d2f_solver *s, const double *x_lin, const double *rhs, double *lam, double *work,
                          const double *tension, double rtol, int32_t max_iter, int32_t warm_start, int32_t *iters,
                          int32_t *status, void *stream) {
    g_err[0] = 0;
    if (!s || !x_lin || !rhs || !lam || !work || !iters || !status)
        return d2f_fail(D2F_EINVAL, "d2f_adjoint_solve: null argument");
    if (s->d.precision != D2F_FP64) return d2f_fail(D2F_EINVAL, "d2f_adjoint_solve: needs an FP64 solver");
    if (s->d.Ne > 0) return d2f_fail(D2F_EINVAL, "d2f_adjoint_solve: IPC contact between bodies has no adjoint tangent");
    if (s->d.n_aff > 0) return d2f_fail(D2F_EINVAL, "d2f_adjoint_solve: affine bodies have no adjoint tangent");
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
