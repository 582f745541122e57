// pncg_kernel.cuh — the implicit step of every scene of a batch, one persistent kernel launch.
//
// GB300 design. A batch is many independent scenes of a few hundred to a few thousand
// nodes. One thread block owns one scene for the whole step: it runs every PNCG iteration
// of that scene (gradient, Dai-Kou direction, curvature, step caps, update) with block
// barriers between phases and deterministic block reductions for the per-scene scalars,
// then pulls the next scene from a queue. A scene's working set (node state, triangle data
// and per-triangle scratch) stays in L1/L2 across its iterations, so HBM sees each scene's
// data about once per step instead of once per phase per iteration, and the ~25 kernel
// launches per iteration of the reference (implicit/solver.py:252-425) become one launch per
// step. Converged scenes retire individually (the reference's convergence poll,
// solver.py:257-259, becomes a per-scene test on the device).
//
// Accumulation into nodes is a gather: a triangle pass writes each corner's gradient and
// Jacobi-diagonal contribution, and a node pass sums its corners in ascending triangle
// order (the reference's serial atomic order) — no atomics on the elastic path.
//
// FP64 budget. GB300 executes FP64 at a small fraction of its FP32 rate, so the element
// routine is written to minimise FP64 operations: J, log J and F^-T are formed once per
// triangle (the reference forms them seven times, kernels.py:85-128), and the six
// directional second derivatives of the Jacobi diagonal use the closed form
//     d2Psi[e_c b^T, e_c b^T] = mu |b|^2 + (la (1 - log J) + mu) ((F^-T b)_c)^2,
// algebraically equal to ddot(dF, nh_d2PsidF2_dir(F, dF)) of core/math.py:84-93 for the
// rank-one dF = e_c b^T of a unit nodal move.
//
// Template parameter R is the element/preconditioner arithmetic type; the library
// instantiates it with double (the mixed-precision step is pncg_mixed_kernel.cuh). This
// header also holds the device code both step kernels share.
#include <cuda_runtime.h>
#include <stdint.h>

#pragma once
#include "../../include/d2f.h"
#include "d2f_math.cuh"

namespace d2f {

constexpr int MAX_COL = 16;
constexpr double BIG = 1.0e30;

template <class R> struct R2T;
template <> struct R2T<double> { using T = double2; };
template <> struct R2T<float> { using T = float2; };
template <class R> struct R4T;
template <> struct R4T<double> { using T = double4_32a; };
template <> struct R4T<float> { using T = float4; };

template <class R> __device__ __forceinline__ typename R2T<R>::T mk2(R a, R b) {
    typename R2T<R>::T v; v.x = a; v.y = b; return v;
}

// ---------------------------------------------------------------------- block reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// ops: 0 sum, 1 max, 2 min. Deterministic: a fixed tree over a fixed thread->data map.
// Result is returned to every thread. `red` holds NW*NV + NV doubles.
template <int NT, int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], const int (&ops)[NV], double *red) {
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double t = ops[k] == 0 ? warp_sum(v[k]) : (ops[k] == 1 ? warp_max(v[k]) : warp_min(v[k]));
        if (lane == 0) red[warp * NV + k] = t;
    }
    block_barrier();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double idv = ops[k] == 0 ? 0.0 : (ops[k] == 1 ? -BIG : BIG);
            double t = lane < NW ? red[lane * NV + k] : idv;
            t = ops[k] == 0 ? warp_sum(t) : (ops[k] == 1 ? warp_max(t) : warp_min(t));
            if (lane == 0) red[NW * NV + k] = t;
        }
    }
    block_barrier();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = red[NW * NV + k];
    block_barrier();
}

// ---------------------------------------------------------------------- per-scene shared state
struct SceneSh {
    double alpha, pHp, gTp, beta, p_inf, clr_min, dE0, gn0, q_inf, alpha_s, dispmax;
    double gPg, g_p, g_Py, y_p, y_Py, gn2;
    double motion, csx, csy, mpx, mpy;  // mixed path: motion since the candidate build, centroid shift
    double dmin_c;                      // smallest candidate-pair distance at the list build (conservative)
    int active, pending, iters, ncand, count, status, rebuild;
};

struct Col {
    int kind;
    double cx, cy, rx, ry, rref, r, mu;
};

// ---------------------------------------------------------------------- small helpers
// Springs._spring (implicit/actuation.py:396-402): d = x_a - x_b, length |d| = sqrt(d.d + 1e-30),
// tension k (|d| - L0), tangential stiffness max(k (1 - L0 / |d|), 0), direction d / |d|.
struct SpringAt {
    double ten, kt, len, nx, ny;
};
__device__ __forceinline__ SpringAt spring_at(double2 xa, double2 xb, double k, double L0) {
    const double dx = xa.x - xb.x, dy = xa.y - xb.y;
    const double ln = sqrt(dx * dx + dy * dy + 1.0e-30);
    const double kt = k * (1.0 - L0 / ln);
    return SpringAt{k * (ln - L0), kt > 0.0 ? kt : 0.0, ln, dx / ln, dy / ln};
}
// the other end of spring k: node sp_b, or the world anchor
__device__ __forceinline__ double2 spring_anchor(const d2f_scene_desc &d, int k) {
    return make_double2(d.sp_anchor[2 * k], d.sp_anchor[2 * k + 1]);
}

__device__ __forceinline__ bool excluded(const d2f_scene_desc &d, int slot, int local) {
    int lo = __ldg(d.excl_ptr + slot), hi = __ldg(d.excl_ptr + slot + 1);
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        int v = __ldg(d.excl_idx + mid);
        if (v == local) return true;
        if (v < local) lo = mid + 1; else hi = mid;
    }
    return false;
}

// ---------------------------------------------------------------------- the step energy
// One thread's share of a scene's step energy (energy_into, solver.py:453-498) in FP64, its
// terms in a fixed order: inertia and external force (kernels.py:445-468, actuation.py:43-50),
// elastic (kernels.py:445-468), collider barriers and lagged friction (core/sdf.py:174-181,
// 274-294; kernels.py:483-513), affine bodies (affine.py:237-246), contact between bodies
// (`ipc`, the caller's pair pass, ipc_contact.py:414-429), springs (actuation.py:447-456),
// pressure (actuation.py:121-130) and tendons (actuation.py:259-268). The thread takes items
// me, me + stride, ... of each list; pos(n) and hat(n) are node n's position and inertial
// target x-hat in FP64. Both kernels call it: the FP64 kernel on its positions, the mixed
// kernel on x_b + r.
template <class Pos, class Hat, class Rm, class B4, class Ipc>
__device__ __forceinline__ double energy_partial(const d2f_scene_desc &d, const d2f_seg &sg, int me, int stride,
                                                 Pos pos, Hat hat, const B4 *Bm, const Rm *Ar, const Rm *Mu,
                                                 const Rm *La, const Col *cols, const double *colmu, Ipc ipc) {
    const double h2 = d.dt * d.dt, inv_dt = 1.0 / d.dt, dhat = d.dhat, kappa = d.kappa, epsv = d.epsv;
    const int n_col = d.n_col;
    const double2 *Xn = reinterpret_cast<const double2 *>(d.xn);
    const double2 *Fx = reinterpret_cast<const double2 *>(d.fext);
    double e = 0.0;
    for (int i = sg.node0 + me; i < sg.node0 + sg.nn; i += stride) {
        const double2 xi = pos(i), xh = hat(i);
        const double ux = xi.x - xh.x, uy = xi.y - xh.y;
        e += 0.5 * d.mass[i] * (ux * ux + uy * uy);
        if (d.fext) {
            const double2 f = Fx[i], xn = Xn[i];
            e += -h2 * (f.x * (xi.x - xn.x) + f.y * (xi.y - xn.y));
        }
    }
    for (int t = sg.tri0 + me; t < sg.tri0 + sg.nt; t += stride) {
        const int i0 = d.tri[3 * t], i1 = d.tri[3 * t + 1], i2 = d.tri[3 * t + 2];
        const double2 x0 = pos(i0), x1 = pos(i1), x2 = pos(i2);
        const B4 B = Bm[t];
        const double e1x = x1.x - x0.x, e1y = x1.y - x0.y, e2x = x2.x - x0.x, e2y = x2.y - x0.y;
        const double F00 = e1x * B.x + e2x * B.z, F01 = e1x * B.y + e2x * B.w;
        const double F10 = e1y * B.x + e2y * B.z, F11 = e1y * B.y + e2y * B.w;
        const double J = F00 * F11 - F10 * F01, logJ = log(dmax(J, 1.0e-6));
        const double I2 = F00 * F00 + F01 * F01 + F10 * F10 + F11 * F11;
        const double mu = (double)Mu[t], la = (double)La[t];
        e += h2 * (double)Ar[t] * (0.5 * mu * (I2 - 2.0) - mu * logJ + 0.5 * la * logJ * logJ);
    }
    for (int j = me; j < sg.nb; j += stride) {
        const int n = d.bnd[sg.bnd0 + j];
        const double2 xi = pos(n);
        const uint8_t fm = d.free_mask[n];
        for (int k = 0; k < n_col; ++k) {
            const Col c = cols[k];
            double dd, nx, ny, gn = 1.0;
            if (c.kind == 0) {
                const double ex = xi.x - c.cx, ey = xi.y - c.cy, dc = sqrt(ex * ex + ey * ey);
                dd = dc - c.r; nx = ex / dc; ny = ey / dc;
            } else {
                const SdfHit hh = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, xi.x, xi.y);
                dd = hh.d;
                gn = sqrt(hh.gx * hh.gx + hh.gy * hh.gy);
                nx = hh.gx / dmax(gn, 1.0e-30); ny = hh.gy / dmax(gn, 1.0e-30);
            }
            if (dd <= 0.0 || dd >= dhat) continue;
            e += h2 * kappa * barrier_b<double>(dd, dhat);
            if (d.friction && (fm & 3)) {
                const double2 xni = Xn[n];
                const double f_n = kappa * dabs(barrier_bp<double>(dd, dhat)) * gn;
                const double vx = (xi.x - xni.x) * inv_dt, vy = (xi.y - xni.y) * inv_dt;
                const double vn = vx * nx + vy * ny;
                const double vtx = vx - vn * nx, vty = vy - vn * ny;
                const double ut = sqrt(vtx * vtx + vty * vty) / inv_dt, a = epsv / inv_dt;
                const double f0 = ut < a ? ut * ut / (2.0 * a) : ut - a * 0.5;
                e += h2 * colmu[k] * f_n * f0;
            }
        }
    }
    for (int b = sg.aff0 + me; b < sg.aff0 + sg.naff; b += stride) {
        const double *q = d.a_q + 6 * b;
        const M2 A{q[1], q[2], q[4], q[5]};
        const double logJ = log(dmax(det2(A), 1.0e-6));
        e += h2 * (0.5 * d.a_Mu[b] * (ddot2(A, A) - 2.0) - d.a_Mu[b] * logJ + 0.5 * d.a_La[b] * logJ * logJ);
    }
    ipc(e);
    for (int k = sg.sp0 + me; k < sg.sp0 + sg.nsp; k += stride) {  // Springs.energy, actuation.py:447-456
        const int b = d.sp_b[k];
        const SpringAt sa = spring_at(pos(d.sp_a[k]), b >= 0 ? pos(b) : spring_anchor(d, k), d.sp_k[k], d.sp_L0[k]);
        const double ext = sa.len - d.sp_L0[k];
        e += 0.5 * h2 * d.sp_k[k] * ext * ext;
    }
    for (int q = sg.pe0 + me; q < sg.pe0 + sg.npe; q += stride) {  // Pressure.energy, actuation.py:121-130
        const int c = d.pe_ch[q];
        const double2 xa = pos(d.pe_a[q]), xb = pos(d.pe_b[q]);
        const double rax = xa.x - d.ch_ref[2 * c], ray = xa.y - d.ch_ref[2 * c + 1];
        const double rbx = xb.x - d.ch_ref[2 * c], rby = xb.y - d.ch_ref[2 * c + 1];
        e += -h2 * d.ch_p[c] * 0.5 * (rax * rby - ray * rbx);
    }
    for (int k = sg.ten0 + me; k < sg.ten0 + sg.nten; k += stride) {
        double L = 0.0;
        for (int j = sg.tent0; j < sg.tent0 + sg.ntent; ++j) {
            if (d.t_tid[j] != k || d.t_nxt[j] < 0) continue;
            const double2 xa = pos(d.t_node[j]), xb = pos(d.t_node[d.t_nxt[j]]);
            const double ex = xb.x - xa.x, ey = xb.y - xa.y;
            L += sqrt(ex * ex + ey * ey);
        }
        if (d.t_stiff[k] > 0.0) {
            const double ext = L - d.t_L0[k];
            if (ext > 0.0) e += 0.5 * h2 * d.t_stiff[k] * ext * ext;
        } else {
            e += h2 * dmax(d.t_Tcmd[k], 0.0) * L;
        }
    }
    return e;
}

// ---------------------------------------------------------------------- the kernel
template <class R, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) pncg_step_kernel(const __grid_constant__ d2f_scene_desc d) {
    using R2 = typename R2T<R>::T;
    using R4 = typename R4T<R>::T;
    constexpr int NW = NT / 32;
    __shared__ SceneSh S;
    __shared__ Col cols[MAX_COL];
    __shared__ double red[NW * 20 + 20];
    __shared__ int sc_next;
    __shared__ int s_wcnt[NW];
    __shared__ unsigned s_wmask[NW];
    __shared__ double s_H6[6][6], s_L6[6][6];
    __shared__ double colmu[MAX_COL];
    extern __shared__ float2 pos32[];  // boundary positions for the candidate-list rebuild

    const int tid = threadIdx.x;
    const double dt = d.dt, h2 = dt * dt, inv_dt = 1.0 / dt;
    const double dhat = d.dhat, kappa = d.kappa, epsv = d.epsv;
    const R rh2 = R(h2), rkappa = R(kappa), rdhat = R(dhat), repsv = R(epsv), rinv_dt = R(inv_dt);
    const bool has_ipc = d.Ne > 0;
    const int n_col = d.n_col;

    double2 *X = reinterpret_cast<double2 *>(d.x);
    double2 *Xn = reinterpret_cast<double2 *>(d.xn);
    double2 *Xh = reinterpret_cast<double2 *>(d.xhat);
    double2 *Vv = reinterpret_cast<double2 *>(d.v);
    R2 *G = reinterpret_cast<R2 *>(d.grad);
    R2 *Gp = reinterpret_cast<R2 *>(d.grad_prev);
    R2 *P = reinterpret_cast<R2 *>(d.p);
    R2 *D = reinterpret_cast<R2 *>(d.diagH);
    R2 *Del = reinterpret_cast<R2 *>(d.diag_el);
    const R4 *Bm = reinterpret_cast<const R4 *>(d.Bm);
    const R *Ar = reinterpret_cast<const R *>(d.area);
    const R *Mu = reinterpret_cast<const R *>(d.mu);
    const R *La = reinterpret_cast<const R *>(d.lam);
    R4 *Esc = reinterpret_cast<R4 *>(d.escr);
    R *Ec = reinterpret_cast<R *>(d.ecache);
    const double2 *Fx = reinterpret_cast<const double2 *>(d.fext);
    const double2 *Tgt = reinterpret_cast<const double2 *>(d.bc_target);
    double2 *Xref = reinterpret_cast<double2 *>(d.xref);
    double2 *Ctr = reinterpret_cast<double2 *>(d.cand_tr);

    if (tid < n_col && tid < MAX_COL) {
        const double *c = d.colliders + 8 * tid;
        cols[tid] = Col{(int)c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7]};
    }

    for (;;) {
        if (tid == 0) sc_next = atomicAdd(d.work, 1);
        block_barrier();
        const int sc = sc_next;
        if (sc >= d.n_scenes) break;
        const d2f_seg sg = d.segs[sc];
        const int n0 = sg.node0, n1 = sg.node0 + sg.nn;
        const int t0 = sg.tri0, t1 = sg.tri0 + sg.nt;
        const bool scene_ipc = has_ipc && sg.ne > 0;
        const bool scene_rig = sg.nrig > 0;
        const int nbl = sg.nb;
        const double near = d.near_factor * dhat;

        // ---- scene-specific collider friction (shared; written before the step-start barrier)
        if (tid < n_col && tid < MAX_COL) colmu[tid] = d.col_mu_env ? d.col_mu_env[sc * n_col + tid] : cols[tid].mu;

        // ================================================================ step setup
        // init_step_kernel (kernels.py:41-50); p = grad = 0 (solver.py:447); none of it for
        // an energy read-out, which takes the state as the last step left it
        const bool eread = d.energy_out != nullptr;
        for (int i = n0 + tid; !eread && i < n1; i += NT) {
            double2 xi = X[i], vi = Vv[i];
            Xn[i] = xi;
            Xh[i] = make_double2(xi.x + dt * d.drag * vi.x, xi.y + dt * d.drag * vi.y);
            G[i] = mk2<R>(R(0), R(0));
            P[i] = mk2<R>(R(0), R(0));
        }
        if (tid == 0) {
            S.active = 1; S.iters = 0; S.dE0 = 0.0; S.status = 0; S.pending = 0;
            S.alpha = d.alpha_max; S.pHp = 0.0; S.q_inf = 0.0; S.alpha_s = 1.0;
            S.ncand = 0; S.rebuild = 1; S.gn0 = 0.0; S.beta = 0.0;
        }
        block_barrier();
        if (!scene_ipc && !eread) {  // apply_bc_kernel, kernels.py:53-59
            for (int b = sg.bc0 + tid; b < sg.bc0 + sg.nbc; b += NT) {
                int n = d.bc_idx[b];
                X[n] = Tgt[b];
                Xh[n] = Tgt[b];
            }
            block_barrier();
        }

        // ---------------------------------------------------------------- contact candidates
        // Node-edge pairs of this scene within reach + skin, rebuilt when a boundary node has
        // moved skin/2 from where the list was built: the pairs closer than `reach` at any
        // later position are then all in the list (each of the three points moves < skin/2).
        // true while every candidate pair is provably out of reach: its distance at the list
        // build (dmin_c, conservative) minus twice the largest node move since then; the pair
        // passes and the ACCD replay would find nothing and are skipped (same result)
        bool ipc_far = false;
        auto ipc_refresh = [&](bool force) {
            double dm = 0.0;
            for (int j = tid; j < nbl; j += NT) {
                double2 xb = X[d.bnd[sg.bnd0 + j]], xr = Xref[sg.bnd0 + j];
                double ex = xb.x - xr.x, ey = xb.y - xr.y;
                dm = dmax(dm, sqrt(ex * ex + ey * ey));
            }
            double v[1] = {dm};
            const int ops[1] = {1};
            block_reduce<NT, 1>(v, ops, red);
            if (!(force || S.rebuild || 2.0 * v[0] >= d.skin)) {
                ipc_far = S.dmin_c - 2.0 * v[0] >= d.reach;
                return;
            }
            // rebuild
            double2 anchor = X[d.bnd[sg.bnd0]];
            for (int j = tid; j < nbl; j += NT) {
                double2 xb = X[d.bnd[sg.bnd0 + j]];
                Xref[sg.bnd0 + j] = xb;
                pos32[j] = make_float2((float)(xb.x - anchor.x), (float)(xb.y - anchor.y));
            }
            if (tid == 0) S.count = 0;
            block_barrier();
            const float rad = (float)(d.reach + d.skin);
            const float slack = 1.0e-5f * rad;
            const long npair = (long)sg.ne * nbl;
            float dmn = 3.0e38f;
            // ordered stream compaction: the list comes out sorted by (edge, boundary slot),
            // the order in which the reference visits the pairs
            for (long base = 0; base < npair; base += NT) {
                const long q = base + tid;
                bool keep = false;
                int k = 0, j = 0;
                if (q < npair) {
                    k = (int)(q / nbl);
                    j = (int)(q - (long)k * nbl);
                    const int ge = sg.edge0 + k;
                    const int a = d.ea[ge], b = d.eb[ge];
                    const int pn = d.bnd[sg.bnd0 + j];
                    if (pn != a && pn != b) {
                        const int la = d.node_bslot[a] - sg.bnd0, lb = d.node_bslot[b] - sg.bnd0;
                        const float2 pa = pos32[la], pb = pos32[lb], pp = pos32[j];
                        // point-segment distance in FP32 with slack: a conservative pre-filter
                        const float abx = pb.x - pa.x, aby = pb.y - pa.y;
                        const float wx = pp.x - pa.x, wy = pp.y - pa.y;
                        float t = (wx * abx + wy * aby) / fmaxf(abx * abx + aby * aby, 1e-30f);
                        t = fminf(fmaxf(t, 0.f), 1.f);
                        const float dx = wx - t * abx, dy = wy - t * aby;
                        const float dd = sqrtf(dx * dx + dy * dy);
                        keep = dd <= rad + slack &&
                               !excluded(d, sg.bnd0 + j, d.ela[ge]) && !excluded(d, sg.bnd0 + j, d.elb[ge]);
                        if (keep) dmn = fminf(dmn, dd);
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                const int lane = tid & 31, warp = tid >> 5;
                if (lane == 0) s_wcnt[warp] = __popc(bal);
                block_barrier();                      // s_wcnt and S.count readable
                int off = S.count + __popc(bal & ((1u << lane) - 1u)), tot = 0;
                for (int w = 0; w < NW; ++w) {
                    if (w < warp) off += s_wcnt[w];
                    tot += s_wcnt[w];
                }
                if (keep && off < sg.ncap) d.cand[sg.cand0 + off] = (int)(((unsigned)k << 16) | (unsigned)j);
                block_barrier();                      // every thread has read them
                if (tid == 0) S.count += tot;         // read after the next chunk's first barrier
            }
            block_barrier();
            double vm[1] = {(double)dmn};
            const int opm[1] = {2};
            block_reduce<NT, 1>(vm, opm, red);
            if (tid == 0) {
                if (S.count > sg.ncap) { S.status = D2F_ECAP; S.ncand = sg.ncap; }
                else S.ncand = S.count;
                S.rebuild = 0;
                S.dmin_c = vm[0] - 1.0e-4 * (double)rad;  // FP32 rounding of the build distances
            }
            block_barrier();
            ipc_far = S.dmin_c >= d.reach;
        };

        // IPC pair evaluation (ipc_pair_kernel + _pair, ipc_contact.py:130-296), FP64.
        // mode 0: gradient + diagonal (atomics into grad/diagH); 1: p^T H p and the ACCD
        // step limit; 3: the kinematic sweep's step limit along the remaining motion.
        auto kin_dir = [&](int n) -> double2 {
            int b = d.node_bc[n];
            if (b < 0) return make_double2(0.0, 0.0);
            double2 t = Tgt[b], x = X[n];
            return make_double2(t.x - x.x, t.y - x.y);
        };
        auto ipc_pairs = [&](int mode, double &acc_pHp, double t_c) {
            if (ipc_far) return;  // every pair out of reach: no term, no cap
            const double idhat = d.ipc_dhat, ikappa = d.ipc_kappa, reach = d.reach, gap = d.gap;
            const double dlo = 1.0e-9 * idhat, onset = 0.02 * idhat;
            const double mu_s = d.friction ? d.ipc_mu : 0.0;
            const int per_body = d.friction ? d.per_body : 0;
            const double floor_ = d.bc_floor * idhat;
            const int nc = S.ncand;
            for (int c = tid; c < nc; c += NT) {
                const unsigned packed = (unsigned)d.cand[sg.cand0 + c];
                const int k = (int)(packed >> 16), j = (int)(packed & 0xffffu);
                int ge = sg.edge0 + k;
                int a = d.ea[ge], b = d.eb[ge], pn = d.bnd[sg.bnd0 + j];
                double2 xa = X[a], xb = X[b], xp = X[pn];
                double abx = xb.x - xa.x, aby = xb.y - xa.y;
                double L2 = dmax(abx * abx + aby * aby, 1.0e-30), Ll = sqrt(L2);
                double wx = xp.x - xa.x, wy = xp.y - xa.y;
                double tt = (wx * abx + wy * aby) / L2;
                double dvx = wx - tt * abx, dvy = wy - tt * aby;
                if (tt <= 0.0) { dvx = wx; dvy = wy; }
                else if (tt >= 1.0) { dvx = xp.x - xb.x; dvy = xp.y - xb.y; }
                double dd = sqrt(dvx * dvx + dvy * dvy);
                if (!(dd < reach)) {
                    if (mode == 1 || mode == 3) Ctr[sg.cand0 + c] = make_double2(1.0e300, 1.0e300);
                    continue;
                }
                if (mode == 1 || mode == 3) {
                    double keep = dmax(gap * dd, idhat - onset);
                    if (dd < idhat) keep = dd - dmin(2.0 * (idhat - dd) + onset, 0.5 * dd);
                    if (mode == 3) keep = dmin(dd, dmax(gap * dd, floor_));
                    double2 qp, qa, qb;
                    if (mode == 3) { qp = kin_dir(pn); qa = kin_dir(a); qb = kin_dir(b); }
                    else {
                        R2 u0 = P[pn], u1 = P[a], u2 = P[b];
                        qp = make_double2(u0.x, u0.y); qa = make_double2(u1.x, u1.y); qb = make_double2(u2.x, u2.y);
                    }
                    double T;
                    const double Rv = accd_profile(xp.x, xp.y, xa.x, xa.y, xb.x, xb.y, qp.x, qp.y,
                                                   qa.x, qa.y, qb.x, qb.y, keep, t_c, T);
                    Ctr[sg.cand0 + c] = make_double2(T, Rv);
                }
                if (mode == 3) continue;
                double mu_p = mu_s;
                if (per_body) {
                    double mi = d.mu_node[pn], mj = d.mu_node[a], sm = mi + mj;
                    mu_p = sm > 0.0 ? 2.0 * mi * mj / sm : 0.0;
                }
                // one barrier-and-friction term (_pair)
                auto term = [&](double coef, int ip, int ia, int ib, double wa, double wb, double dist,
                                double nx, double ny, double ddd) {
                    double bp = barrier_bp<double>(dist, idhat);
                    double f_n = -ikappa * bp;
                    double tnx = -ny, tny = nx;
                    double2 xi = X[ip], xni = Xn[ip], xa_ = X[ia], xna = Xn[ia], xb_ = X[ib], xnb = Xn[ib];
                    double ux = (xi.x - xni.x) - wa * (xa_.x - xna.x) - wb * (xb_.x - xnb.x);
                    double uy = (xi.y - xni.y) - wa * (xa_.y - xna.y) - wb * (xb_.y - xnb.y);
                    double ut = ux * tnx + uy * tny;
                    double vt = dabs(ut) * inv_dt;
                    double kt = mu_p * f_n * inv_dt / dmax(vt, epsv);
                    if (mode == 0) {
                        double bpp = barrier_bpp<double>(dist, idhat);
                        double s = mu_p * f_n * (ut * inv_dt / dmax(vt, epsv));
                        double gx = h2 * (-f_n * nx + s * tnx), gy = h2 * (-f_n * ny + s * tny);
                        double hx = h2 * (ikappa * bpp * nx * nx + kt * tnx * tnx);
                        double hy = h2 * (ikappa * bpp * ny * ny + kt * tny * tny);
                        const int ids[3] = {ip, ia, ib};
                        const double cg[3] = {coef, -coef * wa, -coef * wb};
                        const double ch[3] = {coef, coef * wa * wa, coef * wb * wb};
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            int n = ids[q];
                            uint8_t fm = d.free_mask[n];
                            R *gp_ = reinterpret_cast<R *>(G + n);
                            R *dp_ = reinterpret_cast<R *>(D + n);
                            if (fm & 1) atomicAdd(gp_, R(cg[q] * gx));
                            if (fm & 2) atomicAdd(gp_ + 1, R(cg[q] * gy));
                            atomicAdd(dp_, R(ch[q] * hx));
                            atomicAdd(dp_ + 1, R(ch[q] * hy));
                        }
                    } else if (mode == 2) {  // energy: barrier + lagged friction (ipc_contact.py:414-429)
                        const double asl = epsv / inv_dt, au = dabs(ut);
                        const double f0 = au < asl ? au * au / (2.0 * asl) : au - 0.5 * asl;
                        acc_pHp += coef * h2 * (ikappa * barrier_b<double>(dist, idhat) + mu_p * f_n * f0);
                    } else {
                        double bpp = barrier_bpp<double>(dist, idhat);
                        R2 u0 = P[ip], u1 = P[ia], u2 = P[ib];
                        double qx = double(u0.x) - wa * double(u1.x) - wb * double(u2.x);
                        double qy = double(u0.y) - wa * double(u1.y) - wb * double(u2.y);
                        double dn = qx * nx + qy * ny, dt_ = qx * tnx + qy * tny;
                        double val = dmax(ikappa * (bpp * dn * dn + bp * ddd), 0.0);
                        acc_pHp += coef * h2 * (val + kt * dt_ * dt_);
                    }
                };
                if (tt > 0.0 && tt < 1.0 && dd < idhat) {
                    double dist = dmax(dd, dlo);
                    double ddd = 0.0;
                    if (mode == 1) {
                        R2 pb_ = P[b], pa_ = P[a], pp_ = P[pn];
                        double dex = double(pb_.x) - double(pa_.x), dey = double(pb_.y) - double(pa_.y);
                        double dwx = double(pp_.x) - double(pa_.x), dwy = double(pp_.y) - double(pa_.y);
                        double c0 = abx * wy - aby * wx;
                        double c1 = (dex * wy - dey * wx) + (abx * dwy - aby * dwx);
                        double c2 = 2.0 * (dex * dwy - dey * dwx);
                        double L1 = (abx * dex + aby * dey) / Ll;
                        double Lq = ((dex * dex + dey * dey) - L1 * L1) / Ll;
                        double s0 = c0 / Ll;
                        double s1 = (c1 - s0 * L1) / Ll;
                        ddd = (c2 - 2.0 * s1 * L1 - s0 * Lq) / Ll;
                        if (c0 < 0.0) ddd = -ddd;
                    }
                    term(1.0, pn, a, b, 1.0 - tt, tt, dist, dvx / dist, dvy / dist, ddd);
                }
                double coef_a = -d.ca[ge];
                if (tt <= 0.0) coef_a += 1.0;
                double d_a = sqrt(wx * wx + wy * wy);
                if (coef_a != 0.0 && d_a < idhat) {
                    d_a = dmax(d_a, dlo);
                    double nx = wx / d_a, ny = wy / d_a, ddd = 0.0;
                    if (mode == 1) {
                        R2 pp_ = P[pn], pa_ = P[a];
                        double dwx = double(pp_.x) - double(pa_.x), dwy = double(pp_.y) - double(pa_.y);
                        double dn = dwx * nx + dwy * ny;
                        ddd = ((dwx * dwx + dwy * dwy) - dn * dn) / d_a;
                    }
                    term(coef_a, pn, a, b, 1.0, 0.0, d_a, nx, ny, ddd);
                }
                double coef_b = -d.cb[ge];
                if (tt >= 1.0) coef_b += 1.0;
                double wbx = xp.x - xb.x, wby = xp.y - xb.y;
                double d_b = sqrt(wbx * wbx + wby * wby);
                if (coef_b != 0.0 && d_b < idhat) {
                    d_b = dmax(d_b, dlo);
                    double nx = wbx / d_b, ny = wby / d_b, ddd = 0.0;
                    if (mode == 1) {
                        R2 pp_ = P[pn], pb_ = P[b];
                        double dwx = double(pp_.x) - double(pb_.x), dwy = double(pp_.y) - double(pb_.y);
                        double dn = dwx * nx + dwy * ny;
                        ddd = ((dwx * dwx + dwy * dwy) - dn * dn) / d_b;
                    }
                    term(coef_b, pn, a, b, 0.0, 1.0, d_b, nx, ny, ddd);
                }
            }
        };

        // The reference's serial order for the ACCD cap: each edge reads the cap once, as the
        // edges before it left it, and its pairs lower it (ipc_contact.py:211, 241). Replayed
        // by one thread over the ordered candidate list from the per-pair profiles.
        auto tc_scan = [&](double m0) -> double {  // every thread calls; the result is thread 0's
            if (ipc_far) return m0;  // no pair in reach: every profile is (inf, inf)
            // A pair whose profile threshold T is >= m0 leaves the running minimum untouched at
            // any cap <= m0 (accd_profile: accd(m) = m for m <= T), so only the pairs with
            // T < m0 are replayed — found by warp ballots in candidate order, walked in that
            // order by thread 0 with the same per-edge reset: the result equals the full serial
            // replay.
            double m = m0, t_c = m0;
            int prevk = -1;
            const int nc = S.ncand;
            for (int base = 0; base < nc; base += NT) {
                const int c = base + tid;
                const bool rel = c < nc && Ctr[sg.cand0 + c].x < m0;
                const unsigned bal = __ballot_sync(0xffffffffu, rel);
                if ((tid & 31) == 0) s_wmask[tid >> 5] = bal;
                block_barrier();
                if (tid == 0) {
                    for (int w = 0; w < NW; ++w) {
                        unsigned msk = s_wmask[w];
                        while (msk) {
                            const int cc = base + w * 32 + (__ffs(msk) - 1);
                            msk &= msk - 1;
                            const int k = (int)((unsigned)d.cand[sg.cand0 + cc] >> 16);
                            const double2 pr = Ctr[sg.cand0 + cc];
                            if (k != prevk) { t_c = m; prevk = k; }
                            m = dmin(m, t_c <= pr.x ? t_c : pr.y);
                        }
                    }
                }
                block_barrier();
            }
            return m;
        };

        // kinematic sweep (IPCContact._sweep, ipc_contact.py:456-463 with bc_motion /
        // ccd mode 3 / far cap / bc_advance, :299-331)
        // The scene's step energy at X, FP64, every term (energy_into, solver.py:453-498):
        // inertia and elastic (kernels.py:445-468), collider barriers and lagged friction
        // (core/sdf.py:174-181, 274-294; kernels.py:483-513), external force
        // (actuation.py:43-50), affine bodies (affine.py:237-246), IPC (ipc_contact.py:414-429)
        // and tendons (actuation.py:259-268). Every thread calls; every thread gets the sum.
        auto scene_energy = [&]() -> double {
            double e = energy_partial(d, sg, tid, NT, [&](int n) { return X[n]; }, [&](int n) { return Xh[n]; }, Bm, Ar,
                                      Mu, La, cols, colmu, [&](double &acc) { if (scene_ipc) ipc_pairs(2, acc, 0.0); });
            double v[1] = {e};
            const int ops[1] = {0};
            block_reduce<NT, 1>(v, ops, red);
            return v[0];
        };

        auto sweep = [&]() {
            ipc_refresh(false);
            double qi = 0.0;
            for (int b = sg.bc0 + tid; b < sg.bc0 + sg.nbc; b += NT) {
                double2 q = kin_dir(d.bc_idx[b]);
                qi = dmax(qi, sqrt(q.x * q.x + q.y * q.y));
            }
            double dummy = 0.0;
            ipc_pairs(3, dummy, 1.0);
            double v[1] = {qi};
            const int ops[1] = {1};
            block_reduce<NT, 1>(v, ops, red);
            const double a_tc = tc_scan(1.0);
            if (tid == 0) {
                double a_s = a_tc;
                if (v[0] > 0.0) a_s = dmin(a_s, 0.45 * d.reach / v[0]);
                S.alpha_s = a_s;
            }
            block_barrier();
            const double alpha_s = S.alpha_s;
            for (int b = sg.bc0 + tid; b < sg.bc0 + sg.nbc; b += NT) {
                int n = d.bc_idx[b];
                double2 tg = Tgt[b], x = X[n];
                double2 nx = alpha_s >= 1.0 ? tg : make_double2(x.x + alpha_s * (tg.x - x.x), x.y + alpha_s * (tg.y - x.y));
                X[n] = nx;
                Xh[n] = nx;
            }
            if (tid == 0) S.q_inf = v[0];
            block_barrier();
        };

        if (eread) {  // PNCG2DSolver.energy (solver.py:453-502): every term at x, nothing moved
            if (scene_ipc) ipc_refresh(true);
            const double e = scene_energy();
            if (tid == 0) d.energy_out[sc] = e;
            block_barrier();
            continue;
        }

        if (scene_ipc && sg.nbc > 0) {  // IPCContact.advance_bc, ipc_contact.py:465-473
            sweep();
            if (tid == 0) S.pending = !(S.alpha_s >= 1.0);
            block_barrier();
        }


        // ================================================================ PNCG iterations
        for (int it = 0; it < d.iter_max; ++it) {
            if (scene_ipc && S.pending) {  // IPCContact.before_iteration, ipc_contact.py:475-483
                sweep();
                if (tid == 0) {
                    if (S.q_inf > 0.0) S.active = 1;
                    if (it % 8 == 7) S.pending = !(S.alpha_s >= 1.0);
                }
                block_barrier();
            }
            if (!S.active && !S.pending) break;  // nothing can move this scene any more
            if (S.status != 0) break;

            // ---------------------------------------------- A1: triangle pass (grad + diag)
            for (int t = t0 + tid; t < t1; t += NT) {
                const int i0 = __ldg(d.tri + 3 * t), i1 = __ldg(d.tri + 3 * t + 1), i2 = __ldg(d.tri + 3 * t + 2);
                const R4 B = Bm[t];
                const R A = Ar[t], mu = Mu[t], la = La[t];
                R e1x, e1y, e2x, e2y, G00, G01, G10, G11, c1, P00, P01, P10, P11;
                const double2 x0 = X[i0], x1 = X[i1], x2 = X[i2];
                e1x = R(x1.x - x0.x); e1y = R(x1.y - x0.y); e2x = R(x2.x - x0.x); e2y = R(x2.y - x0.y);
                const R F00 = e1x * B.x + e2x * B.z, F01 = e1x * B.y + e2x * B.w;
                const R F10 = e1y * B.x + e2y * B.z, F11 = e1y * B.y + e2y * B.w;
                const R J = F00 * F11 - F10 * F01;
                const R logJ = rlog<R>(rmax<R>(J, R(1.0e-6)));
                const R iJ = J != R(0) ? R(1) / J : R(0);
                G00 = F11 * iJ; G01 = -F10 * iJ; G10 = -F01 * iJ; G11 = F00 * iJ;  // F^-T
                c1 = la * logJ - mu;
                P00 = mu * F00 + c1 * G00; P01 = mu * F01 + c1 * G01;
                P10 = mu * F10 + c1 * G10; P11 = mu * F11 + c1 * G11;
                const R hA = rh2 * A;
                const R g1x = hA * (P00 * B.x + P01 * B.y), g1y = hA * (P10 * B.x + P11 * B.y);
                const R g2x = hA * (P00 * B.z + P01 * B.w), g2y = hA * (P10 * B.z + P11 * B.w);
                const R kk = la - c1;
                const R b1x = B.x, b1y = B.y, b2x = B.z, b2y = B.w, b0x = -(b1x + b2x), b0y = -(b1y + b2y);
                auto dg = [&](R bx, R by, R &dxo, R &dyo) {
                    R bb = mu * (bx * bx + by * by);
                    R gx = G00 * bx + G01 * by, gy = G10 * bx + G11 * by;
                    dxo = hA * rmax<R>(bb + kk * gx * gx, R(0));
                    dyo = hA * rmax<R>(bb + kk * gy * gy, R(0));
                };
                R d0x, d0y, d1x, d1y, d2x, d2y;
                dg(b0x, b0y, d0x, d0y);
                dg(b1x, b1y, d1x, d1y);
                dg(b2x, b2y, d2x, d2y);
                R4 o0, o1, o2;
                o0.x = -(g1x + g2x); o0.y = -(g1y + g2y); o0.z = d0x; o0.w = d0y;
                o1.x = g1x; o1.y = g1y; o1.z = d1x; o1.w = d1y;
                o2.x = g2x; o2.y = g2y; o2.z = d2x; o2.w = d2y;
                Esc[3 * t] = o0; Esc[3 * t + 1] = o1; Esc[3 * t + 2] = o2;
                R *ec = Ec + 9 * (size_t)t;
                ec[0] = G00; ec[1] = G01; ec[2] = G10; ec[3] = G11; ec[4] = c1;
                ec[5] = e1x; ec[6] = e1y; ec[7] = e2x; ec[8] = e2y;
            }
            block_barrier();

            // ---------------------------------------------- A2: node pass (gather + colliders + friction + force)
            for (int i = n0 + tid; i < n1; i += NT) {
                Gp[i] = G[i];
                const double2 xi = X[i], xh = Xh[i];
                const double m = d.mass[i];
                const uint8_t fm = d.free_mask[i];
                R gx = (fm & 1) ? R(m) * R(xi.x - xh.x) : R(0);
                R gy = (fm & 2) ? R(m) * R(xi.y - xh.y) : R(0);
                R dx = R(m), dy = R(m);
                {
                    // the node's corners, ascending triangle: 8 slots in two vector loads, then
                    // their contributions fetched together (ILP), summed in order
                    const int4 ca = __ldg(reinterpret_cast<const int4 *>(d.inc8) + 2 * i);
                    const int4 cb = __ldg(reinterpret_cast<const int4 *>(d.inc8) + 2 * i + 1);
                    const int cs[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
#pragma unroll
                    for (int h = 0; h < 8; h += 4) {  // two batches of four loads in flight
                        R4 cv[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (cs[h + q] >= 0) cv[q] = Esc[cs[h + q]];
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (cs[h + q] >= 0) { gx += cv[q].x; gy += cv[q].y; dx += cv[q].z; dy += cv[q].w; }
                    }
                    // nodes of more than 8 triangles continue in the CSR
                    const int k0 = __ldg(d.inc_ptr + i) + 8, k1 = __ldg(d.inc_ptr + i + 1);
                    for (int k = k0; k < k1; ++k) {
                        const R4 c = Esc[__ldg(d.inc + k)];
                        gx += c.x; gy += c.y; dx += c.z; dy += c.w;
                    }
                }
                if (scene_rig) Del[i] = mk2<R>(dx, dy);
                if (d.node_bslot[i] >= 0) {
                    // collider barriers: kernels.py:131-157 (disc), core/sdf.py:140-154
                    for (int k = 0; k < n_col; ++k) {
                        const Col c = cols[k];
                        double dd, nx, ny, dc = 1.0;
                        SdfHit hh;
                        if (c.kind == 0) {
                            double ex = xi.x - c.cx, ey = xi.y - c.cy;
                            dc = sqrt(ex * ex + ey * ey);
                            dd = dc - c.r; nx = ex / dc; ny = ey / dc;
                        } else {
                            hh = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, xi.x, xi.y);
                            dd = hh.d; nx = hh.gx; ny = hh.gy;
                        }
                        if (dd <= 0.0 || dd >= dhat) continue;
                        const R rd = R(dd);
                        const R bp = barrier_bp<R>(rd, rdhat), bpp = barrier_bpp<R>(rd, rdhat);
                        const R rnx = R(nx), rny = R(ny);
                        const R s = rh2 * rkappa * bp;
                        gx += s * rnx; gy += s * rny;
                        R hx, hy;
                        if (c.kind == 0) {
                            const R tang = bp / R(dc);
                            hx = rkappa * (bpp * rnx * rnx + tang * (R(1) - rnx * rnx));
                            hy = rkappa * (bpp * rny * rny + tang * (R(1) - rny * rny));
                        } else {
                            hx = rkappa * (bpp * rnx * rnx + bp * R(hh.H00));
                            hy = rkappa * (bpp * rny * rny + bp * R(hh.H11));
                        }
                        dx += rh2 * rmax<R>(hx, R(0));
                        dy += rh2 * rmax<R>(hy, R(0));
                    }
                    // collider friction: kernels.py:640-681 (disc), core/sdf.py:200-233
                    if (d.friction && (fm & 3)) {
                        const double2 xni = Xn[i];
                        for (int k = 0; k < n_col; ++k) {
                            const Col c = cols[k];
                            double dd, nx, ny, gn = 1.0;
                            if (c.kind == 0) {
                                double ex = xi.x - c.cx, ey = xi.y - c.cy, dc = sqrt(ex * ex + ey * ey);
                                dd = dc - c.r; nx = ex / dc; ny = ey / dc;
                            } else {
                                SdfHit h2_ = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, xi.x, xi.y);
                                dd = h2_.d;
                                gn = sqrt(h2_.gx * h2_.gx + h2_.gy * h2_.gy);
                                nx = h2_.gx / dmax(gn, 1.0e-30); ny = h2_.gy / dmax(gn, 1.0e-30);
                            }
                            if (dd <= 0.0 || dd >= dhat) continue;
                            const R rnx = R(nx), rny = R(ny);
                            const R f_n = rkappa * rabs<R>(barrier_bp<R>(R(dd), rdhat)) * R(gn);
                            const R vx = R(xi.x - xni.x) * rinv_dt, vy = R(xi.y - xni.y) * rinv_dt;
                            const R vn = vx * rnx + vy * rny;
                            const R vtx = vx - vn * rnx, vty = vy - vn * rny;
                            const R vtm = rsqrt_<R>(vtx * vtx + vty * vty);
                            const R den = rmax<R>(vtm, repsv);
                            const R mu = R(colmu[k]);
                            const R s = rh2 * mu * f_n;
                            if (fm & 1) gx += s * (vtx / den);
                            if (fm & 2) gy += s * (vty / den);
                            const R kt = s * rinv_dt / den;
                            const R thx = -rny, thy = rnx;
                            if (fm & 1) dx += kt * thx * thx;
                            if (fm & 2) dy += kt * thy * thy;
                        }
                    }
                }
                if (d.fext) {  // ExternalForce, actuation.py:37-41
                    const double2 f = Fx[i];
                    gx -= R(h2 * f.x); gy -= R(h2 * f.y);
                }
                G[i] = mk2<R>(gx, gy);
                D[i] = mk2<R>(dx, dy);
            }
            block_barrier();

            // ---------------------------------------------- A3: contact between bodies, tendons
            if (scene_ipc) {
                ipc_refresh(false);
                double z0 = 0.0;
                ipc_pairs(0, z0, 0.0);
                block_barrier();
            }
            if (sg.nsp > 0 || sg.npe > 0) {
                for (int k = sg.sp0 + tid; k < sg.sp0 + sg.nsp; k += NT) {  // Springs.grad_diag, actuation.py:405-424
                    const int a = d.sp_a[k], b = d.sp_b[k];
                    const SpringAt sa = spring_at(X[a], b >= 0 ? X[b] : spring_anchor(d, k), d.sp_k[k], d.sp_L0[k]);
                    const double gx = h2 * sa.ten * sa.nx, gy = h2 * sa.ten * sa.ny, kk = d.sp_k[k];
                    const double hx = h2 * (kk * sa.nx * sa.nx + sa.kt * (1.0 - sa.nx * sa.nx));
                    const double hy = h2 * (kk * sa.ny * sa.ny + sa.kt * (1.0 - sa.ny * sa.ny));
                    R *ga = reinterpret_cast<R *>(G + a), *da = reinterpret_cast<R *>(D + a);
                    atomicAdd(ga, R(gx)); atomicAdd(ga + 1, R(gy));
                    atomicAdd(da, R(hx)); atomicAdd(da + 1, R(hy));
                    if (b >= 0) {
                        R *gb = reinterpret_cast<R *>(G + b), *db = reinterpret_cast<R *>(D + b);
                        atomicAdd(gb, R(-gx)); atomicAdd(gb + 1, R(-gy));
                        atomicAdd(db, R(hx)); atomicAdd(db + 1, R(hy));
                    }
                }
                for (int e = sg.pe0 + tid; e < sg.pe0 + sg.npe; e += NT) {  // Pressure.grad_diag, actuation.py:98-108
                    const int a = d.pe_a[e], b = d.pe_b[e];
                    const double2 xa = X[a], xb = X[b];
                    const double sp = -0.5 * h2 * d.ch_p[d.pe_ch[e]];
                    const double gx = sp * (xb.y - xa.y), gy = -sp * (xb.x - xa.x);
                    R *ga = reinterpret_cast<R *>(G + a), *gb = reinterpret_cast<R *>(G + b);
                    atomicAdd(ga, R(gx)); atomicAdd(ga + 1, R(gy));
                    atomicAdd(gb, R(gx)); atomicAdd(gb + 1, R(gy));
                }
                block_barrier();
            }
            if (sg.nten > 0) {  // Tendon.grad_diag, actuation.py:169-212, 298-303
                for (int k = sg.ten0 + tid; k < sg.ten0 + sg.nten; k += NT) {
                    double L = 0.0;
                    for (int j = sg.tent0; j < sg.tent0 + sg.ntent; ++j) {
                        if (d.t_tid[j] != k) continue;
                        int m = d.t_nxt[j];
                        if (m < 0) continue;
                        double2 xa = X[d.t_node[j]], xb = X[d.t_node[m]];
                        double ex = xb.x - xa.x, ey = xb.y - xa.y;
                        L += sqrt(ex * ex + ey * ey);
                    }
                    double tau, keff;
                    if (d.t_stiff[k] > 0.0) {
                        double ext = L - d.t_L0[k];
                        tau = ext > 0.0 ? d.t_stiff[k] * ext : 0.0;
                        keff = ext > 0.0 ? d.t_stiff[k] : 0.0;
                    } else {
                        tau = dmax(d.t_Tcmd[k], 0.0); keff = 0.0;
                    }
                    double *ts = d.t_state + 4 * k;
                    ts[0] = L; ts[2] = tau; ts[3] = keff;
                }
                block_barrier();
                for (int j = sg.tent0 + tid; j < sg.tent0 + sg.ntent; j += NT) {
                    int n = d.t_node[j], k = d.t_tid[j];
                    double tau = d.t_state[4 * k + 2], keff = d.t_state[4 * k + 3];
                    double gLx = 0, gLy = 0, geox = 0, geoy = 0;
                    double2 xn_ = X[n];
                    if (d.t_prv[j] >= 0) {
                        double2 xa = X[d.t_node[d.t_prv[j]]];
                        double tx = xn_.x - xa.x, ty = xn_.y - xa.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                        double sx = tx / ln, sy = ty / ln, il = 1.0 / ln;
                        gLx += sx; gLy += sy;
                        geox += (1.0 - sx * sx) * il; geoy += (1.0 - sy * sy) * il;
                    }
                    if (d.t_nxt[j] >= 0) {
                        double2 xb = X[d.t_node[d.t_nxt[j]]];
                        double tx = xb.x - xn_.x, ty = xb.y - xn_.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                        double sx = tx / ln, sy = ty / ln, il = 1.0 / ln;
                        gLx -= sx; gLy -= sy;
                        geox += (1.0 - sx * sx) * il; geoy += (1.0 - sy * sy) * il;
                    }
                    R *gp_ = reinterpret_cast<R *>(G + n);
                    R *dp_ = reinterpret_cast<R *>(D + n);
                    atomicAdd(gp_, R(h2 * tau * gLx));
                    atomicAdd(gp_ + 1, R(h2 * tau * gLy));
                    atomicAdd(dp_, R(h2 * (tau * geox + keff * gLx * gLx)));
                    atomicAdd(dp_ + 1, R(h2 * (tau * geoy + keff * gLy * gLy)));
                }
                block_barrier();
            }

            // ---------------------------------------------- A4: body-level modes gather
            // AffineBodies.gather (affine.py:156-175): J^T g and J^T D J per region
            for (int b = sg.aff0; b < sg.aff0 + sg.naff; ++b) {
                double v[18];
#pragma unroll
                for (int q = 0; q < 18; ++q) v[q] = 0.0;
                for (int k = sg.affn0 + tid; k < sg.affn0 + sg.naffn; k += NT) {
                    if (d.a_grp[k] != b) continue;
                    int i = d.a_node[k];
                    const double *w = d.a_w + 3 * k;
                    R2 g = G[i], dg = D[i];
                    double gx = g.x, gy = g.y, dx = dg.x, dy = dg.y;
                    v[0] += gx * w[0]; v[1] += gx * w[1]; v[2] += gx * w[2];
                    v[3] += gy * w[0]; v[4] += gy * w[1]; v[5] += gy * w[2];
                    const double o[6] = {w[0] * w[0], w[0] * w[1], w[0] * w[2], w[1] * w[1], w[1] * w[2], w[2] * w[2]};
#pragma unroll
                    for (int q = 0; q < 6; ++q) { v[6 + q] += dx * o[q]; v[12 + q] += dy * o[q]; }
                }
                const int ops[18] = {0};
                block_reduce<NT, 18>(v, ops, red);
                if (tid == 0) {
                    for (int q = 0; q < 6; ++q) {
                        d.a_gq_prev[6 * b + q] = d.a_gq[6 * b + q];
                        d.a_gq[6 * b + q] = v[q];
                    }
                    for (int q = 0; q < 12; ++q) d.a_H[18 * b + q] = v[6 + q];
                }
            }
            if (sg.naff > 0) {
                // written by the body entries' threads, read by the nodes' own threads in B1
                block_barrier();
                for (int k = sg.affn0 + tid; k < sg.affn0 + sg.naffn; k += NT) G[d.a_node[k]] = mk2<R>(R(0), R(0));
                block_barrier();
            }
            // RigidModes.gather (affine.py:404-453): centroid, B^T g, B^T g_prev, B^T D' B
            if (tid == 0) { S.gPg = 0.0; S.g_Py = 0.0; S.y_Py = 0.0; }  // (only thread 0 uses these)
            for (int b = sg.rig0; b < sg.rig0 + sg.nrig; ++b) {
                double c[3] = {0.0, 0.0, 0.0};
                for (int k = sg.rign0 + tid; k < sg.rign0 + sg.nrign; k += NT) {
                    if (d.r_grp[k] != b) continue;
                    int i = d.r_node[k];
                    double m = d.mass[i];
                    double2 xi = X[i];
                    c[0] += m * xi.x; c[1] += m * xi.y; c[2] += m;
                }
                const int ops3[3] = {0, 0, 0};
                block_reduce<NT, 3>(c, ops3, red);
                const double cx = c[0] / c[2], cy = c[1] / c[2];
                double v[11];
#pragma unroll
                for (int q = 0; q < 11; ++q) v[q] = 0.0;
                for (int k = sg.rign0 + tid; k < sg.rign0 + sg.nrign; k += NT) {
                    if (d.r_grp[k] != b) continue;
                    int i = d.r_node[k];
                    double2 xi = X[i];
                    double rx = xi.x - cx, ry = xi.y - cy;
                    R2 g = G[i], gp = Gp[i], dg = D[i], de = Del[i];
                    double m = d.mass[i];
                    double dx = dmax(double(dg.x) - double(de.x), 0.0) + m;
                    double dy = dmax(double(dg.y) - double(de.y), 0.0) + m;
                    v[0] += g.x; v[1] += g.y; v[2] += rx * double(g.y) - ry * double(g.x);
                    v[3] += gp.x; v[4] += gp.y; v[5] += rx * double(gp.y) - ry * double(gp.x);
                    v[6] += dx; v[7] += -dx * ry; v[8] += dy; v[9] += dy * rx;
                    v[10] += dx * ry * ry + dy * rx * rx;
                }
                const int ops11[11] = {0};
                block_reduce<NT, 11>(v, ops11, red);
                if (tid == 0) {
                    // inverse of Hc = [[v6, 0, v7], [0, v8, v9], [v7, v9, v10]]
                    double a[9] = {v[6], 0.0, v[7], 0.0, v[8], v[9], v[7], v[9], v[10]};
                    double det = a[0] * (a[4] * a[8] - a[7] * a[5]) - a[1] * (a[3] * a[8] - a[6] * a[5]) +
                                 a[2] * (a[3] * a[7] - a[6] * a[4]);
                    double Hi[9] = {0};
                    if (det != 0.0) {
                        double r = 1.0 / det;
                        Hi[0] = (a[4] * a[8] - a[5] * a[7]) * r; Hi[1] = (a[2] * a[7] - a[1] * a[8]) * r;
                        Hi[2] = (a[1] * a[5] - a[2] * a[4]) * r; Hi[3] = (a[5] * a[6] - a[3] * a[8]) * r;
                        Hi[4] = (a[0] * a[8] - a[2] * a[6]) * r; Hi[5] = (a[2] * a[3] - a[0] * a[5]) * r;
                        Hi[6] = (a[3] * a[7] - a[4] * a[6]) * r; Hi[7] = (a[1] * a[6] - a[0] * a[7]) * r;
                        Hi[8] = (a[0] * a[4] - a[1] * a[3]) * r;
                    }
                    double g[3] = {v[0], v[1], v[2]}, y[3] = {v[0] - v[3], v[1] - v[4], v[2] - v[5]};
                    double z[3], zy[3];
                    for (int r = 0; r < 3; ++r) {
                        z[r] = Hi[3 * r] * g[0] + Hi[3 * r + 1] * g[1] + Hi[3 * r + 2] * g[2];
                        zy[r] = Hi[3 * r] * y[0] + Hi[3 * r + 1] * y[1] + Hi[3 * r + 2] * y[2];
                    }
                    d.r_acc[3 * b] = cx; d.r_acc[3 * b + 1] = cy; d.r_acc[3 * b + 2] = 0.0;
                    for (int r = 0; r < 3; ++r) d.r_zq[3 * b + r] = z[r];
                    // rigid_reduce_kernel (affine.py:456-473): its share of three dot products
                    S.gPg += g[0] * z[0] + g[1] * z[1] + g[2] * z[2];
                    S.g_Py += g[0] * zy[0] + g[1] * zy[1] + g[2] * zy[2];
                    S.y_Py += y[0] * zy[0] + y[1] * zy[1] + y[2] * zy[2];
                }
                block_barrier();
            }

            // ---------------------------------------------- B1: mask + Dai-Kou dot products
            {
                double v[6] = {0, 0, 0, 0, 0, 0};
                for (int i = n0 + tid; i < n1; i += NT) {
                    const uint8_t fm = d.free_mask[i];
                    R2 g = G[i];
                    if (!(fm & 1)) g.x = R(0);
                    if (!(fm & 2)) g.y = R(0);
                    G[i] = g;
                    const R2 dg = D[i], gp = Gp[i], pp = P[i];
                    const R Px = (fm & 1) ? R(1) / rmax<R>(dg.x, R(1.0e-12)) : R(0);
                    const R Py = (fm & 2) ? R(1) / rmax<R>(dg.y, R(1.0e-12)) : R(0);
                    const R yx = g.x - gp.x, yy = g.y - gp.y;
                    const R Pg0 = Px * g.x, Pg1 = Py * g.y, Py0 = Px * yx, Py1 = Py * yy;
                    v[0] += double(g.x * Pg0 + g.y * Pg1);
                    v[1] += double(g.x * pp.x + g.y * pp.y);
                    v[2] += double(g.x * Py0 + g.y * Py1);
                    v[3] += double(yx * pp.x + yy * pp.y);
                    v[4] += double(yx * Py0 + yy * Py1);
                    v[5] += double(g.x * g.x + g.y * g.y);
                }
                const int ops[6] = {0, 0, 0, 0, 0, 0};
                block_reduce<NT, 6>(v, ops, red);
                // ---------------------------------------------- B2: scalars (one thread)
                if (tid == 0) {
                    double gPg = v[0] + S.gPg, g_p = v[1], g_Py = v[2] + S.g_Py, y_p = v[3], y_Py = v[4] + S.y_Py;
                    // affine_reduce_kernel (affine.py:178-205)
                    for (int b = sg.aff0; b < sg.aff0 + sg.naff; ++b) {
                        double *q = d.a_q + 6 * b;
                        M2 A{q[1], q[2], q[4], q[5]};
                        M2 Pm = nh_P(A, d.a_Mu[b], d.a_La[b]);
                        double g[6], y[6], z[6], zy[6];
                        const double hp[6] = {0.0, h2 * Pm.a, h2 * Pm.b, 0.0, h2 * Pm.c, h2 * Pm.d};
                        for (int r = 0; r < 6; ++r) g[r] = d.a_gq[6 * b + r] + hp[r];
                        double (*H)[6] = s_H6, (*L)[6] = s_L6;   // shared: keeps 72 doubles out of registers
                        reduced_hessian(A, d.a_Mu[b], d.a_La[b], h2, d.a_H + 18 * b, H);
                        chol6(H, L);
                        for (int r = 0; r < 6; ++r) y[r] = g[r] - d.a_gq_prev[6 * b + r];
                        chol6_solve(L, g, z);
                        chol6_solve(L, y, zy);
                        const double *pq = d.a_pq + 6 * b;
                        for (int r = 0; r < 6; ++r) {
                            gPg += g[r] * z[r]; g_p += g[r] * pq[r]; g_Py += g[r] * zy[r];
                            y_p += y[r] * pq[r]; y_Py += y[r] * zy[r];
                        }
                        for (int r = 0; r < 6; ++r) { d.a_gq[6 * b + r] = g[r]; d.a_zq[6 * b + r] = z[r]; }
                    }
                    // finalize_beta_kernel (kernels.py:195-217)
                    double bta = 0.0;
                    if (it > 0 && dabs(y_p) > 1.0e-30) bta = g_Py / y_p - y_Py * g_p / (y_p * y_p);
                    double gtp = -gPg + bta * g_p;
                    if (gtp >= 0.0) { bta = 0.0; gtp = -gPg; }
                    // cg_guard_kernel (solver.py:76-94)
                    if (d.cg_guard > 0.0 && it > 0) {
                        double hold = (scene_ipc && S.pending) ? S.q_inf : 0.0;
                        if (hold <= 0.0 && y_p < d.cg_guard * S.alpha * S.pHp) { bta = 0.0; gtp = -gPg; }
                    }
                    S.beta = bta; S.gTp = gtp; S.gn2 = v[5];
                    // affine_direction_kernel (affine.py:208-212)
                    for (int b = sg.aff0; b < sg.aff0 + sg.naff; ++b)
                        for (int r = 0; r < 6; ++r) d.a_pq[6 * b + r] = -d.a_zq[6 * b + r] + bta * d.a_pq[6 * b + r];
                }
                block_barrier();
            }

            // ---------------------------------------------- B3: direction + node curvature and caps
            double acc_pHp = 0.0, acc_pinf = 0.0, acc_clr = BIG, acc_alpha = d.alpha_max;
            {
                const R bta = R(S.beta);
                for (int i = n0 + tid; i < n1; i += NT) {
                    const uint8_t fm = d.free_mask[i];
                    const double2 xi = X[i];
                    R px, py;
                    const int ka = d.node_aff[i];
                    if (ka >= 0) {  // affine_expand_kernel on p_q (affine.py:215-224)
                        const double *w = d.a_w + 3 * ka, *pq = d.a_pq + 6 * d.a_grp[ka];
                        px = R(w[0] * pq[0] + w[1] * pq[1] + w[2] * pq[2]);
                        py = R(w[0] * pq[3] + w[1] * pq[4] + w[2] * pq[5]);
                    } else {  // update_p_kernel (kernels.py:220-230)
                        const R2 g = G[i], dg = D[i], po = P[i];
                        px = (fm & 1) ? -g.x / rmax<R>(dg.x, R(1.0e-12)) + bta * po.x : R(0);
                        py = (fm & 2) ? -g.y / rmax<R>(dg.y, R(1.0e-12)) + bta * po.y : R(0);
                        const int kr = d.node_rig[i];
                        if (kr >= 0) {  // rigid_direction_kernel (affine.py:476-486)
                            const int b = d.r_grp[kr];
                            const double *z = d.r_zq + 3 * b;
                            const double rx = xi.x - d.r_acc[3 * b], ry = xi.y - d.r_acc[3 * b + 1];
                            px -= R(z[0] - z[2] * ry);
                            py -= R(z[1] + z[2] * rx);
                        }
                    }
                    P[i] = mk2<R>(px, py);
                    const double m = d.mass[i];
                    acc_pHp += m * double(px * px + py * py);
                    acc_pinf = dmax(acc_pinf, double(rsqrt_<R>(px * px + py * py)));
                    if (d.node_bslot[i] >= 0) {
                        for (int k = 0; k < n_col; ++k) {
                            const Col c = cols[k];
                            double dd, nx, ny, dc = 1.0, gn = 1.0;
                            SdfHit hh;
                            if (c.kind == 0) {
                                double ex = xi.x - c.cx, ey = xi.y - c.cy;
                                dc = sqrt(ex * ex + ey * ey);
                                dd = dc - c.r; nx = ex / dc; ny = ey / dc;
                                // disc_ccd_kernel (kernels.py:344-371): exact time of impact
                                double a = double(px) * px + double(py) * py;
                                if (a >= 1.0e-24) {
                                    double bq = 2.0 * (ex * px + ey * py), cq = (ex * ex + ey * ey) - c.r * c.r;
                                    double disc = bq * bq - 4.0 * a * cq;
                                    if (disc >= 0.0) {
                                        double sq = sqrt(disc), r1 = (-bq - sq) / (2.0 * a), r2 = (-bq + sq) / (2.0 * a);
                                        double sv = BIG;
                                        if (r1 > 0.0) sv = dmin(sv, r1);
                                        if (r2 > 0.0) sv = dmin(sv, r2);
                                        if (sv < BIG) acc_alpha = dmin(acc_alpha, d.ccd_eta * sv);
                                    }
                                }
                            } else {
                                hh = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, xi.x, xi.y);
                                dd = hh.d; nx = hh.gx; ny = hh.gy;
                                gn = sqrt(nx * nx + ny * ny);
                                // sdf_ccd_kernel (core/sdf.py:297-306): conservative bound
                                double gp = nx * px + ny * py;
                                if (!(gp >= 0.0 || dd <= 0.0)) acc_alpha = dmin(acc_alpha, d.ccd_eta * dd / (-gp));
                            }
                            acc_clr = dmin(acc_clr, dd);
                            if (dd <= 0.0 || dd >= dhat) continue;
                            const R rd = R(dd), rnx = R(nx), rny = R(ny);
                            const R bp = barrier_bp<R>(rd, rdhat), bpp = barrier_bpp<R>(rd, rdhat);
                            R val;
                            if (c.kind == 0) {  // pHp_disc_kernel (kernels.py:276-299)
                                const R pn = px * rnx + py * rny;
                                const R ptx = px - pn * rnx, pty = py - pn * rny;
                                val = rkappa * (bpp * pn * pn + (bp / R(dc)) * (ptx * ptx + pty * pty));
                            } else {  // pHp_sdf_kernel (core/sdf.py:157-171)
                                const R gp = rnx * px + rny * py;
                                const R Hp0 = R(hh.H00) * px + R(hh.H01) * py, Hp1 = R(hh.H10) * px + R(hh.H11) * py;
                                val = rkappa * (bpp * gp * gp + bp * (px * Hp0 + py * Hp1));
                            }
                            acc_pHp += double(rh2 * rmax<R>(val, R(0)));
                            // friction curvature (kernels.py:684-711, core/sdf.py:236-255)
                            if (d.friction && (fm & 3)) {
                                const double2 xni = Xn[i];
                                const R nnx = R(nx / dmax(gn, 1.0e-30)), nny = R(ny / dmax(gn, 1.0e-30));
                                const R f_n = rkappa * rabs<R>(bp) * R(gn);
                                const R vx = R(xi.x - xni.x) * rinv_dt, vy = R(xi.y - xni.y) * rinv_dt;
                                const R vn = vx * nnx + vy * nny;
                                const R vtx = vx - vn * nnx, vty = vy - vn * nny;
                                const R den = rmax<R>(rsqrt_<R>(vtx * vtx + vty * vty), repsv);
                                const R kt = rh2 * R(colmu[k]) * f_n * rinv_dt / den;
                                const R pt = ((fm & 1) ? px : R(0)) * (-nny) + ((fm & 2) ? py : R(0)) * nnx;
                                acc_pHp += double(kt * pt * pt);
                            }
                        }
                    }
                }
            }
            block_barrier();

            // ---------------------------------------------- B4: triangle pass (curvature + inversion cap)
            {
                const R shrink = R(d.area_shrink);
                for (int t = t0 + tid; t < t1; t += NT) {
                    const int i0 = __ldg(d.tri + 3 * t), i1 = __ldg(d.tri + 3 * t + 1), i2 = __ldg(d.tri + 3 * t + 2);
                    const R *ec = Ec + 9 * (size_t)t;
                    const R G00 = ec[0], G01 = ec[1], G10 = ec[2], G11 = ec[3], c1 = ec[4];
                    const R e1x = ec[5], e1y = ec[6], e2x = ec[7], e2y = ec[8];
                    const R2 p0 = P[i0], p1 = P[i1], p2 = P[i2];
                    const R q1x = p1.x - p0.x, q1y = p1.y - p0.y, q2x = p2.x - p0.x, q2y = p2.y - p0.y;
                    const R4 B = Bm[t];
                    const R A = Ar[t], mu = Mu[t], la = La[t];
                    const R f00 = q1x * B.x + q2x * B.z, f01 = q1x * B.y + q2x * B.w;
                    const R f10 = q1y * B.x + q2y * B.z, f11 = q1y * B.y + q2y * B.w;
                    const R dd = f00 * f00 + f01 * f01 + f10 * f10 + f11 * f11;
                    const R GdF = G00 * f00 + G01 * f01 + G10 * f10 + G11 * f11;
                    const R M00 = f00 * G00 + f10 * G10, M01 = f00 * G01 + f10 * G11;
                    const R M10 = f01 * G00 + f11 * G10, M11 = f01 * G01 + f11 * G11;
                    const R tr = M00 * M00 + R(2) * M01 * M10 + M11 * M11;
                    const R val = A * (mu * dd + la * GdF * GdF - c1 * tr);
                    acc_pHp += double(rh2 * rmax<R>(val, R(0)));
                    // inversion_alpha_kernel (kernels.py:303-341)
                    const R a0 = e1x * e2y - e1y * e2x;
                    const R a1 = (e1x * q2y - e1y * q2x) + (q1x * e2y - q1y * e2x);
                    const R a2 = q1x * q2y - q1y * q2x;
                    const R cc = a0 - shrink * a0;
                    if (rabs<R>(a2) < R(1.0e-24)) {
                        if (rabs<R>(a1) > R(1.0e-24)) {
                            const R s = -cc / a1;
                            if (s > R(0)) acc_alpha = dmin(acc_alpha, double(s));
                        }
                    } else {
                        const R disc = a1 * a1 - R(4) * a2 * cc;
                        if (disc >= R(0)) {
                            const R sq = rsqrt_<R>(disc);
                            const R r1 = (-a1 - sq) / (R(2) * a2), r2 = (-a1 + sq) / (R(2) * a2);
                            double s = BIG;
                            if (r1 > R(0)) s = dmin(s, double(r1));
                            if (r2 > R(0)) s = dmin(s, double(r2));
                            if (s < BIG) acc_alpha = dmin(acc_alpha, s);
                        }
                    }
                }
                // affine_pHp_kernel (affine.py:227-234)
                for (int b = sg.aff0 + tid; b < sg.aff0 + sg.naff; b += NT) {
                    const double *q = d.a_q + 6 * b, *pq = d.a_pq + 6 * b;
                    M2 dA{pq[1], pq[2], pq[4], pq[5]}, A{q[1], q[2], q[4], q[5]};
                    acc_pHp += h2 * dmax(ddot2(dA, nh_d2(A, dA, d.a_Mu[b], d.a_La[b])), 0.0);
                }
                // IPC mode 1: curvature along p and the ACCD step limit (t_c = the step cap at
                // the start of the contact pass, alpha_max)
                if (scene_ipc) ipc_pairs(1, acc_pHp, d.alpha_max);
                for (int k = sg.sp0 + tid; k < sg.sp0 + sg.nsp; k += NT) {  // Springs.pHp, actuation.py:427-444
                    const int a = d.sp_a[k], b = d.sp_b[k];
                    const SpringAt sa = spring_at(X[a], b >= 0 ? X[b] : spring_anchor(d, k), d.sp_k[k], d.sp_L0[k]);
                    double dpx = double(P[a].x), dpy = double(P[a].y);
                    if (b >= 0) { dpx -= double(P[b].x); dpy -= double(P[b].y); }
                    const double along = dpx * sa.nx + dpy * sa.ny;
                    acc_pHp += h2 * (d.sp_k[k] * along * along + sa.kt * ((dpx * dpx + dpy * dpy) - along * along));
                }
                for (int e = sg.pe0 + tid; e < sg.pe0 + sg.npe; e += NT) {  // Pressure.pHp, actuation.py:111-118
                    const R2 pa = P[d.pe_a[e]], pb = P[d.pe_b[e]];
                    acc_pHp += -h2 * d.ch_p[d.pe_ch[e]] * (double(pa.x) * double(pb.y) - double(pa.y) * double(pb.x));
                }
                // Tendon.pHp (actuation.py:244-268, 305-310)
                for (int k = sg.ten0 + tid; k < sg.ten0 + sg.nten; k += NT) {
                    double tau = d.t_state[4 * k + 2], keff = d.t_state[4 * k + 3], dL = 0.0;
                    for (int j = sg.tent0; j < sg.tent0 + sg.ntent; ++j) {
                        if (d.t_tid[j] != k) continue;
                        int m = d.t_nxt[j];
                        if (m < 0) continue;
                        int na = d.t_node[j], nb_ = d.t_node[m];
                        double2 xa = X[na], xb = X[nb_];
                        double tx = xb.x - xa.x, ty = xb.y - xa.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                        double sx = tx / ln, sy = ty / ln;
                        R2 pa = P[na], pb = P[nb_];
                        double dpx = double(pb.x) - double(pa.x), dpy = double(pb.y) - double(pa.y);
                        double along = dpx * sx + dpy * sy;
                        dL += along;
                        acc_pHp += h2 * tau * ((dpx * dpx + dpy * dpy) - along * along) * (1.0 / ln);
                    }
                    acc_pHp += h2 * keff * dL * dL;
                }
            }
            {
                double v[4] = {acc_pHp, acc_pinf, acc_clr, acc_alpha};
                const int ops[4] = {0, 1, 2, 2};
                block_reduce<NT, 4>(v, ops, red);
                const double a_ccd = scene_ipc ? tc_scan(d.alpha_max) : 0.0;   // ACCD, reference order
                // ---------------------------------------------- B5: step length and convergence
                if (tid == 0) {
                    const double ph = v[0], pinf = v[1], clr = v[2];
                    double a = v[3];
                    if (scene_ipc) {
                        a = dmin(a, a_ccd);
                        if (pinf > 0.0) a = dmin(a, 0.45 * d.reach / pinf);      // ipc_far_cap_kernel
                    }
                    S.pHp = ph; S.p_inf = pinf; S.clr_min = clr;
                    S.alpha = a;
                    // alpha_finalize_kernel (kernels.py:374-423), plus the optional relative
                    // gradient-norm test
                    if (S.active) {
                        bool done = false;
                        if (d.gtol > 0.0) {
                            if (it == 0) S.gn0 = S.gn2;
                            else if (S.gn2 <= d.gtol * d.gtol * S.gn0) { S.active = 0; done = true; }
                        }
                        if (!done) {
                            if (ph > 0.0) a = dmin(a, -S.gTp / ph);
                            if (clr < near && pinf > 0.0) a = dmin(a, 0.5 * dhat / pinf);
                            if (!(a == a)) { S.status = D2F_ENAN; S.active = 0; S.alpha = 0.0; }
                            else if (a <= 0.0) { S.active = 0; S.alpha = 0.0; }
                            else {
                                S.alpha = a;
                                if (d.tol_x > 0.0 && a * pinf < d.tol_x) { S.active = 0; S.iters += 1; }
                                else {
                                    double dm = -a * S.gTp - 0.5 * a * a * ph;
                                    if (it == 0) S.dE0 = dmax(dm, 1.0e-300);
                                    else if (dm < d.eps * S.dE0) S.active = 0;
                                    S.iters += 1;
                                }
                            }
                        }
                    }
                    // affine_advance_kernel (affine.py:249-257); with the line search the
                    // trial points move q instead (affine_trial_kernel)
                    if (S.active && !d.line_search)
                        for (int b = sg.aff0; b < sg.aff0 + sg.naff; ++b)
                            for (int r = 0; r < 6; ++r) d.a_q[6 * b + r] += S.alpha * d.a_pq[6 * b + r];
                }
                block_barrier();
            }

            // ---------------------------------------------- D1: update x (update_x_kernel + expand),
            // or the backtracking line search (solver.py:397-425)
            if (d.line_search) {
                // E0 at x, then n_backtrack trial points x0 + alpha p, alpha halved while the
                // energy exceeds E0 + ls_tol (|E0| + 1) (ls_halve_kernel, solver.py:63-73)
                // affine bodies: q0 saved after the nodes (AffineBodies.save), the trial
                // q = q0 + alpha p_q and its nodes J q (affine_trial_kernel, affine.py:260-269)
                double2 *__restrict__ X0 = reinterpret_cast<double2 *>(d.xu);
                double *__restrict__ Q0 = d.xu + 2 * (size_t)d.N;
                const double E0 = scene_energy();
                for (int i = n0 + tid; i < n1; i += NT) X0[i] = X[i];
                for (int k = sg.aff0 * 6 + tid; k < (sg.aff0 + sg.naff) * 6; k += NT) Q0[k] = d.a_q[k];
                block_barrier();
                auto trial = [&]() {  // set_x_from_x0_kernel, solver.py:52-60
                    if (S.active) {
                        const double al = S.alpha;
                        for (int k = sg.aff0 * 6 + tid; k < (sg.aff0 + sg.naff) * 6; k += NT)
                            d.a_q[k] = Q0[k] + al * d.a_pq[k];
                        if (sg.naff > 0) block_barrier();
                        for (int i = n0 + tid; i < n1; i += NT) {
                            const int ka = d.node_aff[i];
                            if (ka >= 0) {
                                const double *w = d.a_w + 3 * ka, *q = d.a_q + 6 * d.a_grp[ka];
                                X[i] = make_double2(w[0] * q[0] + w[1] * q[1] + w[2] * q[2],
                                                    w[0] * q[3] + w[1] * q[4] + w[2] * q[5]);
                            } else {
                                const R2 pp = P[i];
                                const double2 x0 = X0[i];
                                X[i] = make_double2(x0.x + al * double(pp.x), x0.y + al * double(pp.y));
                            }
                        }
                    }
                    block_barrier();
                };
                for (int bt = 0; bt < d.n_backtrack; ++bt) {
                    trial();
                    if (scene_ipc) ipc_refresh(false);
                    const double E = scene_energy();
                    if (tid == 0 && S.active && E > E0 + d.ls_tol * (dabs(E0) + 1.0)) S.alpha *= 0.5;
                    block_barrier();
                }
                trial();
            } else {
                const bool act = S.active != 0;
                const double al = S.alpha;
                for (int i = n0 + tid; i < n1; i += NT) {
                    const int ka = d.node_aff[i];
                    double2 nx;
                    if (ka >= 0) {
                        const double *w = d.a_w + 3 * ka, *q = d.a_q + 6 * d.a_grp[ka];
                        nx = make_double2(w[0] * q[0] + w[1] * q[1] + w[2] * q[2], w[0] * q[3] + w[1] * q[4] + w[2] * q[5]);
                    } else if (act) {
                        const R2 pp = P[i];
                        const double2 xi = X[i];
                        nx = make_double2(xi.x + al * double(pp.x), xi.y + al * double(pp.y));
                    } else {
                        continue;
                    }
                    X[i] = nx;
                }
                block_barrier();
            }
        }

        // ================================================================ commit_v_kernel (kernels.py:437-441)
        for (int i = n0 + tid; i < n1; i += NT) {
            const double2 xi = X[i], xn = Xn[i];
            Vv[i] = make_double2((xi.x - xn.x) * inv_dt, (xi.y - xn.y) * inv_dt);
        }
        if (tid == 0) {
            d.iters[sc] = S.iters;
            d.active[sc] = S.active;
            d.status[sc] = S.status;
        }
        block_barrier();
    }
}

}  // namespace d2f


// Launch shapes the library is built with: (threads per scene block, minimum resident
// blocks per SM the register budget is fitted to). d2f_scene_desc.threads / blocks_per_sm
// select one; the autotuner (tune.py) measures them.
#define D2F_VARIANTS(X) X(32, 16) X(64, 8) X(128, 4) X(256, 2) X(256, 3)

namespace d2f {
// one translation unit per precision instantiates the variants (pncg_fp64.cu, pncg_mixed.cu)
cudaError_t launch_fp64(int nt, int minb, const d2f_scene_desc &d, int grid, int smem, cudaStream_t st);
cudaError_t launch_mixed(int nt, int minb, const d2f_scene_desc &d, int grid, int smem, cudaStream_t st);
int occupancy_fp64(int nt, int minb, int smem);
int occupancy_mixed(int nt, int minb, int smem, int feat);
// The mixed batch kernel's feature sets. Bit 0: contact between bodies (IPC); bit 1: affine
// bodies, tendons, springs, pressure and the line search. A batch runs the smallest set that
// covers it: code for terms a batch does not have still costs registers, and the batch kernel
// runs at 80-128 registers a thread, where the live values the rare paths add spill in the
// hot loop (measured at 256 threads: a 736-byte stack frame with every term, 240 without
// bit 1, 32 with neither). Instantiated in pncg_mixed.cu (all) and pncg_mixed_feat.cu.
enum : int { FEAT_IPC = 1, FEAT_RARE = 2, FEAT_ALL = 3 };
inline int mixed_features(const d2f_scene_desc &d) {
    int f = d.Ne > 0 ? FEAT_IPC : 0;
    if (d.n_aff > 0 || d.n_ten > 0 || d.n_sp > 0 || d.n_pe > 0 || d.line_search) f = FEAT_ALL;
    return f;
}
cudaError_t launch_mixed_feat(int feat, int nt, int minb, const d2f_scene_desc &d, int grid, int smem, cudaStream_t st);
int occupancy_mixed_feat(int feat, int nt, int minb, int smem);
// threads per block of the cluster path (a block per SM: 16 warps to hide the latency of a
// large scene's passes, 128 registers a thread)
constexpr int kClusterThreads = 512;
// the mixed kernel with a cluster of cs (8, 12 or 16) kClusterThreads-thread blocks per scene
// (pncg_mixed_cluster.cu): grid = clusters x cs blocks; max_clusters_mixed = the clusters
// that fit on the device at once (0: that cluster size cannot be launched)
cudaError_t launch_mixed_cluster(int cs, const d2f_scene_desc &d, int grid, int smem, cudaStream_t st);
int max_clusters_mixed(int cs, int smem);
// every SM on one scene (pncg_mixed_cluster.cu): a cooperative launch of `grid` blocks of
// kClusterThreads, one per SM; grid_blocks_mixed = the blocks that can be co-resident
cudaError_t launch_mixed_grid(const d2f_scene_desc &d, int grid, int smem, cudaStream_t st);
int grid_blocks_mixed(int smem);
int grid_max_blocks();
}  // namespace d2f
