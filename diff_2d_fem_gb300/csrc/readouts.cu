// readouts.cu — per-element strain and stress of a configuration (core/fields.py), on the
// device: one thread per triangle, FP64.
//
//   F = Ds B                                   (Ds: edge vectors as columns, B = Dm^-1)
//   E = (F^T F - I) / 2,  E_zz = 0             Green-Lagrange strain (plane strain)
//   sigma = (mu F F^T + (lam ln J - mu) I) / J, sigma_zz = lam ln J / J   (Neo-Hookean Cauchy)
//   von Mises: strain sqrt(2/3 e':e'), stress sqrt(3/2 s':s')  (' deviatoric, 3 x 3)
//   signed: the in-plane principal value of larger magnitude, with its sign
#include <cuda_runtime.h>
#include <stdint.h>

#include "d2f_solver.h"

namespace {

// deviatoric squared norm of the 3 x 3 tensor [[a, b, 0], [b, d, 0], [0, 0, z]]
__device__ __forceinline__ double dev_norm2(double a, double b, double d, double z) {
    const double m = (a + d + z) / 3.0;
    const double da = a - m, dd = d - m, dz = z - m;
    return da * da + dd * dd + dz * dz + 2.0 * b * b;
}

// in-plane principal value of larger magnitude of [[a, b], [b, d]]
__device__ __forceinline__ double signed_principal(double a, double b, double d) {
    const double m = 0.5 * (a + d), r = sqrt(0.25 * (a - d) * (a - d) + b * b);
    const double hi = m + r, lo = m - r;
    return fabs(hi) >= fabs(lo) ? hi : lo;
}

__global__ void element_fields_kernel(int T, const int32_t *__restrict__ tri, const double *__restrict__ Bm,
                                      const double *__restrict__ mu, const double *__restrict__ lam,
                                      const double *__restrict__ x, double *strain_vm, double *strain_signed,
                                      double *stress_vm, double *stress_signed) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
        const int i0 = tri[3 * t], i1 = tri[3 * t + 1], i2 = tri[3 * t + 2];
        const double e1x = x[2 * i1] - x[2 * i0], e1y = x[2 * i1 + 1] - x[2 * i0 + 1];
        const double e2x = x[2 * i2] - x[2 * i0], e2y = x[2 * i2 + 1] - x[2 * i0 + 1];
        const double b00 = Bm[4 * t], b01 = Bm[4 * t + 1], b10 = Bm[4 * t + 2], b11 = Bm[4 * t + 3];
        const double F00 = e1x * b00 + e2x * b10, F01 = e1x * b01 + e2x * b11;
        const double F10 = e1y * b00 + e2y * b10, F11 = e1y * b01 + e2y * b11;
        // Green-Lagrange strain
        const double E00 = 0.5 * (F00 * F00 + F10 * F10 - 1.0), E11 = 0.5 * (F01 * F01 + F11 * F11 - 1.0);
        const double E01 = 0.5 * (F00 * F01 + F10 * F11);
        if (strain_vm) strain_vm[t] = sqrt(2.0 / 3.0 * dev_norm2(E00, E01, E11, 0.0));
        if (strain_signed) strain_signed[t] = signed_principal(E00, E01, E11);
        if (stress_vm || stress_signed) {
            const double J = F00 * F11 - F01 * F10;
            const double lnJ = log(J > 1.0e-12 ? J : 1.0e-12);
            const double m = mu[t], l = lam[t], c = l * lnJ - m;
            const double S00 = (m * (F00 * F00 + F01 * F01) + c) / J, S11 = (m * (F10 * F10 + F11 * F11) + c) / J;
            const double S01 = m * (F00 * F10 + F01 * F11) / J, Szz = l * lnJ / J;
            if (stress_vm) stress_vm[t] = sqrt(1.5 * dev_norm2(S00, S01, S11, Szz));
            if (stress_signed) stress_signed[t] = signed_principal(S00, S01, S11);
        }
    }
}

}  // namespace

extern "C" int32_t d2f_element_fields(int32_t T, const int32_t *tri, const double *Bm, const double *mu,
                                      const double *lam, const double *x, double *strain_vm,
                                      double *strain_signed, double *stress_vm, double *stress_signed,
                                      void *stream) {
    g_err[0] = 0;
    if (T <= 0 || !tri || !Bm || !x) return d2f_fail(D2F_EINVAL, "d2f_element_fields: empty mesh or null input");
    if ((stress_vm || stress_signed) && (!mu || !lam))
        return d2f_fail(D2F_EINVAL, "d2f_element_fields: stress needs mu and lam");
    const int threads = 256;
    int blocks = (T + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    element_fields_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(T, tri, Bm, mu, lam, x, strain_vm, strain_signed,
                                                                       stress_vm, stress_signed);
    if (cudaGetLastError() != cudaSuccess) return d2f_fail(D2F_ECUDA, "d2f_element_fields: launch failed");
    return D2F_OK;
}

// ============================================================================ contact forces
// Contact read-outs at the solver's current positions x, with the slip of the last step
// measured from x_n (PNCG2DSolver.contact_force / collider_force, implicit/solver.py:553-612):
//   what 0: the force contact exerts ON every node (N x 2): the colliders' barrier (flag 1)
//           and the contact between bodies (flag 2), with friction (flag 4); every DOF, the
//           kinematic ones included (the reaction a prescribed body feels);
//   what 1: the reaction ON collider `col` (all colliders when col < 0) per scene (B x 2):
//           the barrier (kernels.py:517-530, core/sdf.py:185-191), with friction (flag 4;
//           kernels.py:724-743, core/sdf.py:259-271 — as the reference, the disc adds
//           +mu f_n tdir and the other shapes -mu f_n tdir).
#include "pncg_kernel.cuh"

namespace {

constexpr int kReadThreads = 256;

__device__ __forceinline__ void add2(double *out, int n, double fx, double fy) {
    atomicAdd(out + 2 * n, fx);
    atomicAdd(out + 2 * n + 1, fy);
}

__global__ void __launch_bounds__(kReadThreads) contact_force_kernel(const __grid_constant__ d2f_scene_desc d,
                                                                     int what, int col, int flags, double *out) {
    using namespace d2f;
    __shared__ Col cols[MAX_COL];
    __shared__ double red[2 * (kReadThreads / 32) + 2];
    const int tid = threadIdx.x;
    if (tid < d.n_col && tid < MAX_COL) {
        const double *c = d.colliders + 8 * tid;
        cols[tid] = Col{(int)c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7]};
    }
    block_barrier();
    const double2 *X = reinterpret_cast<const double2 *>(d.x);
    const double2 *Xn = reinterpret_cast<const double2 *>(d.xn);
    const double dhat = d.dhat, kappa = d.kappa, inv_dt = 1.0 / d.dt, epsv = d.epsv;
    const bool rub = (flags & 4) && d.friction;
    for (int sc = blockIdx.x; sc < d.n_scenes; sc += gridDim.x) {
        const d2f_seg sg = d.segs[sc];
        double rx = 0.0, ry = 0.0;  // what 1: this thread's share of the reaction
        if (what == 1 || (flags & 1)) {
            for (int j = tid; j < sg.nb; j += kReadThreads) {
                const int n = d.bnd[sg.bnd0 + j];
                const double2 xi = X[n], xni = Xn[n];
                for (int k = 0; k < d.n_col; ++k) {
                    if (what == 1 && col >= 0 && k != col) continue;
                    const Col c = cols[k];
                    double dd, gx, gy, gn = 1.0;  // distance, its gradient, |gradient|
                    if (c.kind == 0) {
                        const double ex = xi.x - c.cx, ey = xi.y - c.cy, dc = sqrt(ex * ex + ey * ey);
                        dd = dc - c.r; gx = ex / dc; gy = ey / dc;
                    } else {
                        const SdfHit h = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, xi.x, xi.y);
                        dd = h.d; gx = h.gx; gy = h.gy; gn = sqrt(gx * gx + gy * gy);
                    }
                    if (dd <= 0.0 || dd >= dhat) continue;
                    const double bp = barrier_bp<double>(dd, dhat);
                    double fx = -kappa * bp * gx, fy = -kappa * bp * gy;  // barrier force on the node
                    double tx = 0.0, ty = 0.0;                          // friction force on the node
                    if (rub) {
                        const double mu = d.col_mu_env ? d.col_mu_env[sc * d.n_col + k] : c.mu;
                        const double nx = gx / dmax(gn, 1.0e-30), ny = gy / dmax(gn, 1.0e-30);
                        const double f_n = kappa * dabs(bp) * gn;
                        const double vx = (xi.x - xni.x) * inv_dt, vy = (xi.y - xni.y) * inv_dt;
                        const double vn = vx * nx + vy * ny, vtx = vx - vn * nx, vty = vy - vn * ny;
                        const double den = dmax(sqrt(vtx * vtx + vty * vty), epsv);
                        tx = -mu * f_n * vtx / den;
                        ty = -mu * f_n * vty / den;
                        if (what == 1 && c.kind != 0) { tx = -tx; ty = -ty; }
                    }
                    if (what == 0) {
                        add2(out, n, fx + tx, fy + ty);
                    } else {
                        rx += -fx - tx;
                        ry += -fy - ty;
                    }
                }
            }
        }
        if (what == 1) {  // per-scene sum in a fixed tree
            double v[2] = {rx, ry};
            const int ops[2] = {0, 0};
            block_reduce<kReadThreads, 2>(v, ops, red);
            if (tid == 0) { out[2 * sc] = v[0]; out[2 * sc + 1] = v[1]; }
            continue;
        }
        if (!(flags & 2) || d.Ne <= 0 || sg.ne <= 0) continue;
        // contact between bodies: every edge-node pair of the scene within dhat, the terms of
        // the IPC gradient (_pair, ipc_contact.py:130-296) with h^2 = 1, on every DOF
        const double idhat = d.ipc_dhat, ikappa = d.ipc_kappa, dlo = 1.0e-9 * idhat;
        const double mu_s = ((flags & 4) && d.friction) ? d.ipc_mu : 0.0;
        const int per_body = ((flags & 4) && d.friction) ? d.per_body : 0;
        for (int k = tid; k < sg.ne; k += kReadThreads) {
            const int ge = sg.edge0 + k;
            const int a = d.ea[ge], b = d.eb[ge];
            const double2 xa = X[a], xb = X[b];
            const double abx = xb.x - xa.x, aby = xb.y - xa.y;
            const double L2 = dmax(abx * abx + aby * aby, 1.0e-30);
            for (int j = 0; j < sg.nb; ++j) {
                const int pn = d.bnd[sg.bnd0 + j];
                if (pn == a || pn == b) continue;
                const double2 xp = X[pn];
                const double wx = xp.x - xa.x, wy = xp.y - xa.y;
                const double tt = (wx * abx + wy * aby) / L2;
                double dvx = wx - tt * abx, dvy = wy - tt * aby;
                if (tt <= 0.0) { dvx = wx; dvy = wy; }
                else if (tt >= 1.0) { dvx = xp.x - xb.x; dvy = xp.y - xb.y; }
                const double dd = sqrt(dvx * dvx + dvy * dvy);
                if (!(dd < idhat)) continue;
                if (excluded(d, sg.bnd0 + j, d.ela[ge]) || excluded(d, sg.bnd0 + j, d.elb[ge])) continue;
                double mu_p = mu_s;
                if (per_body) {
                    const double mi = d.mu_node[pn], mj = d.mu_node[a], sm = mi + mj;
                    mu_p = sm > 0.0 ? 2.0 * mi * mj / sm : 0.0;
                }
                auto term = [&](double coef, double wa, double wb, double dist, double nx, double ny) {
                    const double f_n = -ikappa * barrier_bp<double>(dist, idhat);
                    const double tnx = -ny, tny = nx;
                    const double2 xnp = Xn[pn], xna = Xn[a], xnb = Xn[b];
                    const double ux = (xp.x - xnp.x) - wa * (xa.x - xna.x) - wb * (xb.x - xnb.x);
                    const double uy = (xp.y - xnp.y) - wa * (xa.y - xna.y) - wb * (xb.y - xnb.y);
                    const double ut = ux * tnx + uy * tny, vt = dabs(ut) * inv_dt;
                    const double s = mu_p * f_n * (ut * inv_dt / dmax(vt, epsv));
                    const double gx = -f_n * nx + s * tnx, gy = -f_n * ny + s * tny;
                    add2(out, pn, -coef * gx, -coef * gy);
                    if (wa != 0.0) add2(out, a, coef * wa * gx, coef * wa * gy);
                    if (wb != 0.0) add2(out, b, coef * wb * gx, coef * wb * gy);
                };
                if (tt > 0.0 && tt < 1.0) {
                    const double dist = dmax(dd, dlo);
                    term(1.0, 1.0 - tt, tt, dist, dvx / dist, dvy / dist);
                }
                double coef_a = -d.ca[ge];
                if (tt <= 0.0) coef_a += 1.0;
                double d_a = sqrt(wx * wx + wy * wy);
                if (coef_a != 0.0 && d_a < idhat) {
                    d_a = dmax(d_a, dlo);
                    term(coef_a, 1.0, 0.0, d_a, wx / d_a, wy / d_a);
                }
                double coef_b = -d.cb[ge];
                if (tt >= 1.0) coef_b += 1.0;
                const double wbx = xp.x - xb.x, wby = xp.y - xb.y;
                double d_b = sqrt(wbx * wbx + wby * wby);
                if (coef_b != 0.0 && d_b < idhat) {
                    d_b = dmax(d_b, dlo);
                    term(coef_b, 0.0, 1.0, d_b, wbx / d_b, wby / d_b);
                }
            }
        }
    }
}

}  // namespace

extern "C" int32_t d2f_contact_force(d2f_solver *s, int32_t what, int32_t collider, int32_t flags, double *out,
                                     void *stream) {
    g_err[0] = 0;
    if (!s || !out) return d2f_fail(D2F_EINVAL, "d2f_contact_force: null argument");
    if (what != 0 && what != 1) return d2f_fail(D2F_EINVAL, "d2f_contact_force: what must be 0 (nodes) or 1 (collider)");
    if (what == 1 && collider >= s->d.n_col) return d2f_fail(D2F_EINVAL, "d2f_contact_force: no such collider");
    cudaStream_t st = (cudaStream_t)stream;
    if (what == 0 && cudaMemsetAsync(out, 0, sizeof(double) * 2 * (size_t)s->d.N, st) != cudaSuccess)
        return d2f_fail(D2F_ECUDA, "d2f_contact_force: cudaMemsetAsync failed");
    int blocks = s->d.n_scenes < 152 * 8 ? s->d.n_scenes : 152 * 8;
    contact_force_kernel<<<blocks, kReadThreads, 0, st>>>(s->d, what, collider, flags, out);
    if (cudaGetLastError() != cudaSuccess) return d2f_fail(D2F_ECUDA, "d2f_contact_force: launch failed");
    return D2F_OK;
}
