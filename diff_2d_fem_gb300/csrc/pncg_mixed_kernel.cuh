// pncg_mixed_kernel.cuh — the mixed-precision implicit step: FP32 iterations on small offsets
// from an FP64 base state, FP64 where the reference's accuracy argument needs it.
//
// GB300 executes FP64 at ~1/64 of its FP32 rate, so in this path an iteration performs
// (almost) no FP64 instruction:
//
//   * the base: positions x = x_b + r with x_b an FP64 base state and r an FP32 offset, and
//     the gradient g = g0 + (g - g0) with g0 the elastic, tendon and external forces at x_b
//     evaluated in FP64 and kept as a compensated FP32 pair. The base starts at x_n (the
//     state at the start of the step) and is rebuilt every REBASE iterations (x_b += r,
//     r = 0, g0 at the new x_b), so r and the increments shrink as the solve converges:
//     neither the FP32 resolution of the positions nor the large, mutually cancelling forces
//     of a loaded body bound how far it converges (iterative refinement);
//   * triangles: F = I + Hn + K, Hn = dU0 B with dU0 the FP64 edge differences of
//     (x_b - X_rest) rounded once per rebuild, K = (r-differences) B; the gradient takes the
//     stress increment P(F) - P(Fn) in a form without cancellation, the diagonal and the
//     curvature the stress at F;
//   * inertia: x - x_hat = dx - dt e^(-dt c) v with dx = (x_b - x_n) + r in FP32;
//   * half-space colliders: phi = phi0 + n.dx with phi0 = n.(x_n - c) in FP64 per step,
//     so the barrier distance keeps FP64 accuracy near contact; other collider shapes,
//     tendons and affine bodies evaluate in FP64 from x_b + r;
//   * contact between bodies: each candidate pair's geometry relative to one of its nodes
//     (FP64 differences of the base positions, rounded once, plus the FP32 offsets), its
//     barrier, friction and ACCD profile in FP32; a pair with a term closer than 1e-3 d-hat
//     (the barrier near its singularity) in FP64;
//   * friction: slip velocity dx / dt;
//   * rigid modes: arms a = (x_n - c_n) + dx - (c - c_n).
//   * dot products: each thread accumulates its FP32 products with compensated (TwoSum)
//     FP32 pairs, warps and then the per-warp partials merge the pairs, and each sum is
//     converted to FP64 once. The Dai-Kou beta, the step length and the energy-decrease test
//     stay FP64 (divisions through an FP32 reciprocal and one FP64 Newton step);
//   * step caps (inversion, CCD, |p|, clearance), the gradient-norm test and the rigid-mode
//     preconditioner's 3x3 solve are FP32;
//   * the line search (when on): every energy term in FP64 at x_b + r.
// At the end of the step x = x_b + r and v = (x - x_n)/dt in FP64.
#pragma once
#include <cooperative_groups.h>
#include <type_traits>

#include "pncg_kernel.cuh"

namespace d2f {

// ---------------------------------------------------------------------- compensated FP32 sums
struct FF {
    float hi, lo;
};
__device__ __forceinline__ void ff_add(FF &a, float b) {  // Knuth TwoSum
    const float s = a.hi + b;
    const float bp = s - a.hi;
    const float err = (a.hi - (s - bp)) + (b - bp);
    a.hi = s;
    a.lo += err;
}
__device__ __forceinline__ FF ff_merge(FF a, FF b) {
    const float s = a.hi + b.hi;
    const float bp = s - a.hi;
    const float err = (a.hi - (s - bp)) + (b.hi - bp);
    const float lo = err + a.lo + b.lo;
    const float hi = s + lo;
    return FF{hi, lo - (hi - s)};
}

// Block reduction: NS compensated sums (returned as FP64) and NM FP32 reductions
// (ops 0 = plain sum, 1 = max, 2 = min). Deterministic. `fred` holds NW*(2*NS+NM) floats,
// `dres` NS doubles, `mres` NM floats.
template <int NT, int NS, int NM>
__device__ __forceinline__ void block_reduce_mx(FF (&s)[NS], float (&m)[NM], const int (&mops)[NM],
                                                double (&out_s)[NS], float (&out_m)[NM], float *fred,
                                                double *dres, float *mres) {
    static_assert(NS <= 20 && NM <= 16 && 2 * NS + NM <= 40, "fred / dres / mres of the step kernel");
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            FF b{__shfl_down_sync(0xffffffffu, s[k].hi, o), __shfl_down_sync(0xffffffffu, s[k].lo, o)};
            s[k] = ff_merge(s[k], b);
        }
#pragma unroll
        for (int k = 0; k < NM; ++k) {
            const float b = __shfl_down_sync(0xffffffffu, m[k], o);
            m[k] = mops[k] == 1 ? fmaxf(m[k], b) : mops[k] == 2 ? fminf(m[k], b) : m[k] + b;
        }
    }
    if (lane == 0) {
        float *w = fred + warp * (2 * NS + NM);
#pragma unroll
        for (int k = 0; k < NS; ++k) { w[2 * k] = s[k].hi; w[2 * k + 1] = s[k].lo; }
#pragma unroll
        for (int k = 0; k < NM; ++k) w[2 * NS + k] = m[k];
    }
    block_barrier();
    // the per-warp partials. Sum k: its NW pairs converted to FP64 (exactly) by NW adjacent
    // lanes, q = lane within the group, and added in a fixed shuffle tree, so the FP64 sum
    // costs one conversion and log2(NW) dependent additions (dependent FP64 operations are
    // slow on this part); extremum j by thread SOFF + j (small blocks: thread j, after its sum).
    {
        constexpr int SOFF = ((NS * NW + 31) / 32) * 32;
        const int t = threadIdx.x;
        if (t < SOFF) {
            const int k = t / NW, q = t % NW;
            double v = 0.0;
            if (t < NS * NW) v = (double)fred[q * (2 * NS + NM) + 2 * k] + (double)fred[q * (2 * NS + NM) + 2 * k + 1];
#pragma unroll
            for (int o = NW / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (q == 0 && t < NS * NW) dres[k] = v;
        }
        const int j = SOFF + NM <= NT ? t - SOFF : t;
        if (j >= 0 && j < NM) {
            float a = fred[2 * NS + j];
            for (int q = 1; q < NW; ++q) {
                const float b = fred[q * (2 * NS + NM) + 2 * NS + j];
                a = mops[j] == 1 ? fmaxf(a, b) : mops[j] == 2 ? fminf(a, b) : a + b;
            }
            mres[j] = a;
        }
    }
    block_barrier();
#pragma unroll
    for (int k = 0; k < NS; ++k) out_s[k] = dres[k];
#pragma unroll
    for (int k = 0; k < NM; ++k) out_m[k] = mres[k];
    // no barrier here: a later call writes `fred` only after its threads passed this call's
    // second barrier (every read of `fred` is before it), and `dres` / `mres` only after its own
    // first barrier, which every thread reaches after reading this call's results
}

// ---------------------------------------------------------------------- every SM on one scene
// The grid mode (CS == 0): all blocks of one cooperative launch, one per SM, work on one scene
// at a time. Blocks exchange through global memory, a part of the mixed step's scratch: a
// barrier header, then per block a reduction slot (two alternating buffers), a list-count slot
// and an ordered list of the candidates below the running cap (GX_REL of them: a block with
// more sends the replay to its full walk, as a cluster block past REL_CAP does).
// the multi-block paths' ACCD replay: candidates below the running cap, per block
constexpr int REL_CAP = 512;
constexpr int GX_RED = 20;          // doubles per block per reduction buffer
constexpr int GX_REL = 64;          // ordered candidates per block
constexpr int GX_MAX_BLOCKS = 256;  // blocks (SMs) the exchange is sized for
struct GridX {
    unsigned *count, *gen;
    int *err;
    double *red;   // [2][nb][GX_RED]
    int *cnt;      // [nb]
    int *nrel;     // [nb]
    int *rel;      // [nb][GX_REL]
    int nb, parity;
};
__host__ __device__ inline size_t grid_exchange_bytes(int nb) {
    return 256 + (size_t)2 * nb * GX_RED * sizeof(double) + (size_t)nb * (2 + GX_REL) * sizeof(int);
}
__device__ inline GridX grid_exchange(void *base, int nb) {
    unsigned char *b = static_cast<unsigned char *>(base);
    GridX g;
    g.count = reinterpret_cast<unsigned *>(b);
    g.gen = reinterpret_cast<unsigned *>(b) + 1;
    g.err = reinterpret_cast<int *>(b) + 2;
    g.red = reinterpret_cast<double *>(b + 256);
    g.cnt = reinterpret_cast<int *>(g.red + (size_t)2 * nb * GX_RED);
    g.nrel = g.cnt + nb;
    g.rel = g.nrel + nb;
    g.nb = nb;
    g.parity = 0;
    return g;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Every block of the launch (co-resident: a cooperative launch). Thread 0 of each block
// arrives on a counter; the last one resets it and advances the generation the others wait
// for. The wait is bounded (2 s): past it the block sets the shared error flag and every later
// barrier returns at once, so a fault in the protocol ends the kernel with an error status
// instead of hanging the device.
static __device__ __noinline__ void grid_barrier(GridX &g) {
    block_barrier();
    if (threadIdx.x == 0 && !*reinterpret_cast<volatile int *>(g.err)) {
        const unsigned gen0 = ld_acquire_u32(g.gen);
        __threadfence();
        if (atomicAdd(g.count, 1u) == (unsigned)g.nb - 1u) {
            atomicExch(g.count, 0u);
            __threadfence();
            atomicAdd(g.gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (ld_acquire_u32(g.gen) == gen0) {
                if (*reinterpret_cast<volatile int *>(g.err)) break;
                if (global_ns() - t0 > 2000000000ull) {
                    atomicExch(g.err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    block_barrier();
}

// Reductions over the thread group working on one scene. CS == 1: the block reduction. A
// cluster of CS blocks on one scene (large scenes): the block reduction, then the CS block
// results combined in rank order through distributed shared memory, so every block of the
// cluster holds the same, deterministic result. `cres` / `cmres`: per-block scratch.
template <int NT, int CS, int NV>
__device__ __forceinline__ void scene_reduce(double (&v)[NV], const int (&ops)[NV], double *red, double *cres,
                                             GridX *gx = nullptr) {
    static_assert(NV <= 20, "red / cres of the step kernel");
    block_reduce<NT, NV>(v, ops, red);
    if constexpr (CS == 0) {  // every block's result through global memory, combined in block order
        constexpr int NW = NT / 32;
        double *buf = gx->red + (size_t)gx->parity * gx->nb * GX_RED;
        gx->parity ^= 1;  // the next reduction writes the other buffer: no barrier after the reads
        if (threadIdx.x < NV) buf[(size_t)blockIdx.x * GX_RED + threadIdx.x] = red[NW * NV + threadIdx.x];
        grid_barrier(*gx);
        if (threadIdx.x < NV) {
            const int k = threadIdx.x;
            double a = buf[k];
            for (int r = 1; r < gx->nb; ++r) {
                const double b = buf[(size_t)r * GX_RED + k];
                a = ops[k] == 0 ? a + b : (ops[k] == 1 ? dmax(a, b) : dmin(a, b));
            }
            cres[k] = a;
        }
        block_barrier();
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = cres[k];
    } else if constexpr (CS > 1) {
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
        constexpr int NW = NT / 32;
        double *mine = red + NW * NV;  // the block result, kept by block_reduce
        cluster_barrier();
        if (threadIdx.x < NV) {
            const int k = threadIdx.x;
            double a = cl.map_shared_rank(mine, 0)[k];
            for (int r = 1; r < CS; ++r) {
                const double b = cl.map_shared_rank(mine, r)[k];
                a = ops[k] == 0 ? a + b : (ops[k] == 1 ? dmax(a, b) : dmin(a, b));
            }
            cres[k] = a;
        }
        cluster_barrier();  // cres ready, and every remote read of `red` done before it is reused
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = cres[k];
    }
}

template <int NT, int CS, int NS, int NM>
__device__ __forceinline__ void scene_reduce_mx(FF (&s)[NS], float (&m)[NM], const int (&mops)[NM],
                                                double (&out_s)[NS], float (&out_m)[NM], float *fred,
                                                double *dres, float *mres, double *cres, float *cmres,
                                                GridX *gx = nullptr) {
    block_reduce_mx<NT, NS, NM>(s, m, mops, out_s, out_m, fred, dres, mres);
    if constexpr (CS == 0) {  // every block's sums and extrema through global memory, in block order
        static_assert(NS + NM <= GX_RED, "grid reduction slot");
        double *buf = gx->red + (size_t)gx->parity * gx->nb * GX_RED;
        gx->parity ^= 1;
        const int k = threadIdx.x;
        if (k < NS) buf[(size_t)blockIdx.x * GX_RED + k] = dres[k];
        else if (k < NS + NM) buf[(size_t)blockIdx.x * GX_RED + k] = (double)mres[k - NS];
        grid_barrier(*gx);
        if (k < NS) {
            double a = 0.0;
            for (int r = 0; r < gx->nb; ++r) a += buf[(size_t)r * GX_RED + k];
            cres[k] = a;
        } else if (k < NS + NM) {
            const int j = k - NS;
            float a = (float)buf[k];
            for (int r = 1; r < gx->nb; ++r) {
                const float b = (float)buf[(size_t)r * GX_RED + k];
                a = mops[j] == 1 ? fmaxf(a, b) : mops[j] == 2 ? fminf(a, b) : a + b;
            }
            cmres[j] = a;
        }
        block_barrier();
#pragma unroll
        for (int q = 0; q < NS; ++q) out_s[q] = cres[q];
#pragma unroll
        for (int q = 0; q < NM; ++q) out_m[q] = cmres[q];
    } else if constexpr (CS > 1) {
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
        cluster_barrier();
        const int k = threadIdx.x;
        if (k < NS) {
            double a = 0.0;
            for (int r = 0; r < CS; ++r) a += cl.map_shared_rank(dres, r)[k];
            cres[k] = a;
        } else if (k < NS + NM) {
            const int j = k - NS;
            float a = cl.map_shared_rank(mres, 0)[j];
            for (int r = 1; r < CS; ++r) {
                const float b = cl.map_shared_rank(mres, r)[j];
                a = mops[j] == 1 ? fmaxf(a, b) : mops[j] == 2 ? fminf(a, b) : a + b;
            }
            cmres[j] = a;
        }
        cluster_barrier();
#pragma unroll
        for (int q = 0; q < NS; ++q) out_s[q] = cres[q];
#pragma unroll
        for (int q = 0; q < NM; ++q) out_m[q] = cmres[q];
    }
}

// Byte layout of the mixed path's per-step scratch (d2f_scene_desc.mscr), 256-aligned parts.
struct MixedLayout {
    size_t xd, hvm, g0, gd, xbd, xr, db, rarm, ninfo, du0, phi0, rcs, pb, gx, total;
};
__host__ __device__ inline MixedLayout mixed_layout(long N, long T, long Nb, long n_col, long n_rig) {
    auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
    MixedLayout L;
    size_t o = 0;
    L.xd = o; o = up(o + (size_t)N * 8);
    L.hvm = o; o = up(o + (size_t)N * 16);
    L.g0 = o; o = up(o + (size_t)N * 16);
    L.gd = o; o = up(o + (size_t)N * 16);
    L.xbd = o; o = up(o + (size_t)N * 16);
    L.xr = o; o = up(o + (size_t)N * 8);
    L.db = o; o = up(o + (size_t)N * 8);
    L.rarm = o; o = up(o + (size_t)N * 8);
    L.ninfo = o; o = up(o + (size_t)N * 8);
    L.du0 = o; o = up(o + (size_t)T * 16);
    L.phi0 = o; o = up(o + (size_t)N * (n_col > 0 ? n_col : 1) * 4);
    L.rcs = o; o = up(o + (size_t)(n_rig > 0 ? n_rig : 1) * 8);
    L.pb = o; o = up(o + (size_t)(Nb > 0 ? Nb : 1) * 8);
    L.gx = o; o = up(o + grid_exchange_bytes(GX_MAX_BLOCKS));  // the all-SM mode's block exchange
    L.total = o;
    return L;
}

// d len / d x at eyelet node n of a tendon (prv / nxt: neighbouring eyelet entries or -1),
// FP64 positions from pos(node)
template <class PosF>
__device__ __forceinline__ double2 tendon_dlen(PosF pos, const int32_t *t_node, int prv, int nxt, int n) {
    double gx = 0.0, gy = 0.0;
    const double2 xn = pos(n);
    if (prv >= 0) {
        const double2 xa = pos(t_node[prv]);
        const double tx = xn.x - xa.x, ty = xn.y - xa.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
        gx += tx / ln; gy += ty / ln;
    }
    if (nxt >= 0) {
        const double2 xb = pos(t_node[nxt]);
        const double tx = xb.x - xn.x, ty = xb.y - xn.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
        gx -= tx / ln; gy -= ty / ln;
    }
    return make_double2(gx, gy);
}

// iterations between rebuilds of the FP64 gradient base
constexpr int REBASE = 64;
// packed per-node flags (NINFO.x): bits 0-1 free mask, then these, bits 4-7 the rigid piece
constexpr int NI_AFF = 4, NI_RIG = 8;
// contact candidate lists of scenes with at least HASH_MIN_NB boundary nodes on a cluster are
// built through a spatial hash of HASH_B buckets (every other scene tests all edge-node pairs)
constexpr int HASH_MIN_NB = 4096, HASH_B = 4096;
// the hash (HASH_B bucket ends + the slots, 4 bytes each) reuses the 8 bytes per boundary node
// of dynamic shared memory the exhaustive build holds its positions in
static_assert(HASH_MIN_NB >= HASH_B, "hash tables must fit the boundary-position buffer");

// AffineBodies.gather (affine.py:156-175) for bodies b0, b0 + stride, ... < b1: a warp per
// body over the body's own nodes (lane of 32), J^T g and J^T D J summed in a fixed shuffle
// tree (FP64). Out of line: its 18 accumulators would otherwise weigh on the register
// allocation of the whole step kernel, in which affine bodies are a rare path. (Plain
// pointers, not the descriptor: a reference to it would copy it into every thread's stack.)
static __device__ __noinline__ void affine_gather(const int32_t *a_ptr, const int32_t *a_node, const double *a_w,
                                                  const float2 *G, const float2 *D, double *a_gq, double *a_gq_prev,
                                                  double *a_H, int b0, int b1, int stride, int lane) {
    for (int b = b0; b < b1; b += stride) {
        double v[18];
#pragma unroll
        for (int q = 0; q < 18; ++q) v[q] = 0.0;
        const int k1 = a_ptr[b + 1];
        for (int k = a_ptr[b] + lane; k < k1; k += 32) {
            const int i = a_node[k];
            const double *w = a_w + 3 * k;
            const float2 g = G[i], dg = D[i];
            const double gx = g.x, gy = g.y, dx = dg.x, dy = dg.y;
            v[0] += gx * w[0]; v[1] += gx * w[1]; v[2] += gx * w[2];
            v[3] += gy * w[0]; v[4] += gy * w[1]; v[5] += gy * w[2];
            const double o[6] = {w[0] * w[0], w[0] * w[1], w[0] * w[2], w[1] * w[1], w[1] * w[2], w[2] * w[2]};
#pragma unroll
            for (int q = 0; q < 6; ++q) { v[6 + q] += dx * o[q]; v[12 + q] += dy * o[q]; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int q = 0; q < 18; ++q) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
        }
        if (lane == 0) {
            for (int q = 0; q < 6; ++q) {
                a_gq_prev[6 * b + q] = a_gq[6 * b + q];
                a_gq[6 * b + q] = v[q];
            }
            for (int q = 0; q < 12; ++q) a_H[18 * b + q] = v[6 + q];
        }
    }
}

// affine_reduce_kernel (affine.py:178-205) for bodies b0, b0 + stride, ... < b1: each body's
// 6x6 solve by this thread (FP64), its five Dai-Kou terms added to ab (g.z, g.p, g.zy, y.p,
// y.zy). Out of line for the same reason as affine_gather.
static __device__ __noinline__ void affine_solve(const double *a_q, const double *a_Mu, const double *a_La,
                                                 double *a_gq, const double *a_gq_prev, const double *a_H,
                                                 const double *a_pq, double *a_zq, double h2, int b0, int b1,
                                                 int stride, double *ab) {
    for (int b = b0; b < b1; b += stride) {
        const double *q = a_q + 6 * b;
        const M2 A{q[1], q[2], q[4], q[5]};
        const M2 Pm = nh_P(A, a_Mu[b], a_La[b]);
        double g[6], y[6], z[6], zy[6], H[6][6], L[6][6];
        const double hp[6] = {0.0, h2 * Pm.a, h2 * Pm.b, 0.0, h2 * Pm.c, h2 * Pm.d};
        for (int r = 0; r < 6; ++r) g[r] = a_gq[6 * b + r] + hp[r];
        reduced_hessian(A, a_Mu[b], a_La[b], h2, a_H + 18 * b, H);
        chol6(H, L);
        for (int r = 0; r < 6; ++r) y[r] = g[r] - a_gq_prev[6 * b + r];
        chol6_solve(L, g, z);
        chol6_solve(L, y, zy);
        const double *pq = a_pq + 6 * b;
        for (int r = 0; r < 6; ++r) {
            ab[0] += g[r] * z[r]; ab[1] += g[r] * pq[r]; ab[2] += g[r] * zy[r];
            ab[3] += y[r] * pq[r]; ab[4] += y[r] * zy[r];
        }
        for (int r = 0; r < 6; ++r) { a_gq[6 * b + r] = g[r]; a_zq[6 * b + r] = z[r]; }
    }
}

// ---------------------------------------------------------------------- the kernel
// Device pointers of the per-step scratch parts (host-computed from d2f_scene_desc.mscr).
struct MixedPtrs {
    float2 *xd, *rarm, *xr, *db, *pb, *rcs;
    float4 *hvm, *g0, *gd, *du0;
    double2 *g0d, *xbd;
    int2 *ninfo;
    float *phi0;
    unsigned char *gx;
};
inline MixedPtrs mixed_ptrs(const d2f_scene_desc &d) {
    const MixedLayout L = mixed_layout(d.N, d.T, d.Nb, d.n_col, d.n_rig);
    unsigned char *ms = static_cast<unsigned char *>(d.mscr);
    MixedPtrs p;
    p.xd = reinterpret_cast<float2 *>(ms + L.xd);
    p.rarm = reinterpret_cast<float2 *>(ms + L.rarm);
    p.xr = reinterpret_cast<float2 *>(ms + L.xr);
    p.db = reinterpret_cast<float2 *>(ms + L.db);
    p.pb = reinterpret_cast<float2 *>(ms + L.pb);
    p.rcs = reinterpret_cast<float2 *>(ms + L.rcs);
    p.hvm = reinterpret_cast<float4 *>(ms + L.hvm);
    p.g0 = reinterpret_cast<float4 *>(ms + L.g0);
    p.gd = reinterpret_cast<float4 *>(ms + L.gd);
    p.du0 = reinterpret_cast<float4 *>(ms + L.du0);
    p.g0d = reinterpret_cast<double2 *>(ms + L.g0);
    p.xbd = reinterpret_cast<double2 *>(ms + L.xbd);
    p.ninfo = reinterpret_cast<int2 *>(ms + L.ninfo);
    p.phi0 = reinterpret_cast<float *>(ms + L.phi0);
    p.gx = ms + L.gx;
    return p;
}

// The mixed kernel's per-scene FP32 scalars: FP32 copies of the step length and Dai-Kou
// coefficient for the node passes, the rigid-mode preconditioner's terms, the caps and the
// gradient-norm test. A chain of dependent FP64 operations on one thread costs ~100 cycles an
// operation on this part, and these run once per iteration while the scene's other threads
// wait at the next barrier; the CG coefficients themselves and the energy-decrease test stay
// FP64 (SceneSh).
struct SceneF {
    float alpha, beta, pinf, gn0, gn2;
    float gPg, g_Py, y_Py;      // the rigid pieces' Dai-Kou terms
    float csx, csy, mpx, mpy;   // single rigid piece: centroid shift (copy of SceneSh's), sum m p / M
    float inv_m;                // single rigid piece: 1 / M
};

// 1 / v in FP64 from the FP32 reciprocal and one Newton step (relative error ~1e-14): four
// FP64 operations where a division takes several times that, on a thread the scene's other
// warps wait for. Outside FP32's range, the division.
__device__ __forceinline__ double rcp64(double v) {
    const float f = (float)v;
    if (!(fabsf(f) > 1.0e-36f && fabsf(f) < 1.0e36f)) return 1.0 / v;
    const double r = (double)(1.0f / f);
    return r * fma(-v, r, 2.0);
}

// One rigid piece's preconditioner solve (RigidModes reduce, rigid_reduce_kernel,
// affine.py:456-473) in FP32: v = B^T g (3), B^T g_prev (3) and the symmetric 3x3 B^T D' B as
// a00, a02, a11, a12, a22 (a01 = 0); z = A^-1 B^T g and zy = A^-1 B^T (g - g_prev) through the
// adjugate (A^-1 = 0 for a singular A, as the FP64 kernel); the piece's Dai-Kou terms g.z,
// g.zy, y.zy added to F; z to zq (FP64) or zf.
__device__ __forceinline__ void rigid_precondition(const float *v, SceneF &F, double *zq, float *zf) {
    const float A = v[6], B = v[7], C = v[8], D = v[9], E = v[10];
    const float c00 = C * E - D * D, c01 = B * D, c02 = -B * C;
    const float c11 = A * E - B * B, c12 = -A * D, c22 = A * C;
    const float det = A * c00 + B * c02;
    const float r = det != 0.f ? 1.f / det : 0.f;
    const float g0 = v[0], g1 = v[1], g2 = v[2];
    const float y0 = g0 - v[3], y1 = g1 - v[4], y2 = g2 - v[5];
    const float z0 = (c00 * g0 + c01 * g1 + c02 * g2) * r;
    const float z1 = (c01 * g0 + c11 * g1 + c12 * g2) * r;
    const float z2 = (c02 * g0 + c12 * g1 + c22 * g2) * r;
    const float w0 = (c00 * y0 + c01 * y1 + c02 * y2) * r;
    const float w1 = (c01 * y0 + c11 * y1 + c12 * y2) * r;
    const float w2 = (c02 * y0 + c12 * y1 + c22 * y2) * r;
    if (zq) { zq[0] = z0; zq[1] = z1; zq[2] = z2; }
    if (zf) { zf[0] = z0; zf[1] = z1; zf[2] = z2; }
    F.gPg += g0 * z0 + g1 * z1 + g2 * z2;
    F.g_Py += g0 * w0 + g1 * w1 + g2 * w2;
    F.y_Py += y0 * w0 + y1 * w1 + y2 * w2;
}

// CS: blocks per scene. 1: a block per scene (batches). > 1: a cluster of CS blocks works on
// one scene (large scenes): the scene's loops are spread over the cluster's threads, phases are
// separated by cluster barriers, reductions combine the blocks' results through distributed
// shared memory, and the per-scene scalars are kept, identically, by every block.
// FEAT: the terms the kernel is compiled with (FEAT_IPC, FEAT_RARE; mixed_features).
template <int NT, int MINB, int CS = 1, int FEAT = FEAT_ALL>
__global__ void __launch_bounds__(NT, MINB) pncg_mixed_kernel(const __grid_constant__ d2f_scene_desc d,
                                                              const __grid_constant__ MixedPtrs mp) {
    namespace cg = cooperative_groups;
    constexpr int NW = NT / 32;
    constexpr bool GR = CS == 0;   // every block of the launch on one scene (cooperative launch)
    constexpr bool CLU = CS > 1;   // a thread-block cluster on one scene
    constexpr bool CL = CS != 1;   // several blocks on one scene (either form)
    const int NBS = GR ? (int)gridDim.x : CS;  // blocks working on one scene
    const int GS = NBS * NT;                   // threads working on one scene
    __shared__ SceneSh S;
    __shared__ SceneF F;
    __shared__ Col cols[MAX_COL];
    __shared__ double red[NW * 20 + 20];
    __shared__ float fred[NW * 40];
    __shared__ double dres[20];
    __shared__ float mres[16];               // block_reduce_mx: up to 16 FP32 results (rigid pass: 12)
    __shared__ int sc_next;
    __shared__ int s_cnt;                    // cluster list build: this block's kept pairs
    __shared__ int s_nrel;                   // cluster ACCD replay: this block's pairs below the cap
    __shared__ int s_rel[REL_CAP];           // ... their candidate indices, in order
    __shared__ double cres[24];              // cluster reductions: the combined result
    __shared__ float cmres[16];
    __shared__ int s_wcnt[NW];
    __shared__ unsigned s_wmask[NW];
    __shared__ double colmu[MAX_COL];
    __shared__ double s_H6[6][6], s_L6[6][6];  // the batch kernel's affine 6x6 solve (thread 0)
    __shared__ float s_zf[8][3], s_cs[8][2];  // rigid-mode correction of up to 8 pieces, FP32
    __shared__ float colf[MAX_COL][2], colmuf[MAX_COL];  // half-space normals, friction (FP32)
    extern __shared__ float2 pos32[];

    const int tid = threadIdx.x;
    int crank = 0;
    if constexpr (GR) crank = (int)blockIdx.x;
    else if constexpr (CLU) crank = (int)cg::this_cluster().block_rank();
    const int gt = crank * NT + tid;  // this thread's index among the scene's threads
    GridX gxv{};
    if constexpr (GR) gxv = grid_exchange(mp.gx, (int)gridDim.x);
    GridX *const gxp = GR ? &gxv : nullptr;
    auto gsync = [&]() {              // a phase barrier of the scene's thread group
        if constexpr (GR) grid_barrier(gxv);
        else if constexpr (CLU) cluster_barrier();
        else block_barrier();
    };
    const double dt = d.dt, h2 = dt * dt, inv_dt = 1.0 / dt;
    const double dhat = d.dhat;
    const float fh2 = (float)h2, fkappa = (float)d.kappa, fdhat = (float)dhat, fepsv = (float)d.epsv,
                finv_dt = (float)inv_dt, feta = (float)d.ccd_eta;
    constexpr bool F_IPC = (FEAT & FEAT_IPC) != 0, F_RARE = (FEAT & FEAT_RARE) != 0;
    const bool has_ipc = F_IPC && d.Ne > 0;
    const bool line_search = F_RARE && d.line_search;
    const int n_col = d.n_col;
    // the stop tests' and caps' constants in FP32
    const bool use_gtol = d.gtol > 0.0, use_tolx = d.tol_x > 0.0, use_guard = d.cg_guard > 0.0;
    const float fgtol2 = (float)(d.gtol * d.gtol), ftol_x = (float)d.tol_x;
    const float falpha_max = (float)d.alpha_max, fnear = (float)(d.near_factor * dhat), freach45 = (float)(0.45 * d.reach);

    double2 *__restrict__ X = reinterpret_cast<double2 *>(d.x);
    double2 *__restrict__ Xn = reinterpret_cast<double2 *>(d.xn);
    double2 *__restrict__ Vv = reinterpret_cast<double2 *>(d.v);
    float2 *__restrict__ G = reinterpret_cast<float2 *>(d.grad);
    float2 *__restrict__ Gp = reinterpret_cast<float2 *>(d.grad_prev);
    float2 *__restrict__ P = reinterpret_cast<float2 *>(d.p);
    float2 *__restrict__ D = reinterpret_cast<float2 *>(d.diagH);
    float2 *__restrict__ Del = reinterpret_cast<float2 *>(d.diag_el);
    const float4 *__restrict__ Bm = reinterpret_cast<const float4 *>(d.Bm);
    const float *__restrict__ Ar = reinterpret_cast<const float *>(d.area);
    const float *__restrict__ Mu = reinterpret_cast<const float *>(d.mu);
    const float *__restrict__ La = reinterpret_cast<const float *>(d.lam);
    const double2 *__restrict__ Fx = reinterpret_cast<const double2 *>(d.fext);
    const double2 *__restrict__ Tgt = reinterpret_cast<const double2 *>(d.bc_target);
    double2 *__restrict__ Ctr = reinterpret_cast<double2 *>(d.cand_tr);
    // rest edge vectors of each triangle (X1 - X0, X2 - X0 after any active-strain change)
    const double2 *__restrict__ Dm2 = reinterpret_cast<const double2 *>(d.Dm);
    // the per-step scratch arrays: pointers from the parameter space (constant bank), not
    // registers
    float2 *__restrict__ XD = mp.xd;       // x - x_n
    float4 *__restrict__ HVM = mp.hvm;     // x_hat - x_n, mass
    float4 *__restrict__ G0 = mp.g0;       // step-start gradient, FP32 pair
    double2 *__restrict__ G0d = mp.g0d;    // the same, FP64 while it is built
    double2 *__restrict__ Esc64 = reinterpret_cast<double2 *>(d.escr);  // per-corner FP64 forces (base builds)
    float4 *__restrict__ GD = mp.gd;       // per node: elastic gradient + diagonal sums
    float2 *__restrict__ RARM = mp.rarm;   // x_n - c_n (rigid pieces)
    int2 *__restrict__ NINFO = mp.ninfo;   // node flags, boundary slot
    float4 *__restrict__ DU0 = mp.du0;     // displacement edges at the base x_b
    double2 *__restrict__ XBd = mp.xbd;    // base positions x_b (FP64)
    float2 *__restrict__ XR = mp.xr;       // x - x_b
    float2 *__restrict__ DB = mp.db;       // x_b - x_n
    float *__restrict__ PHI0 = mp.phi0;    // half-space distances at x_n, per node
    float2 *__restrict__ PB = mp.pb;       // boundary positions at the list build (hashed scenes)
    float2 *__restrict__ RCS = mp.rcs;     // rigid pieces: centroid shift

    if (tid < n_col && tid < MAX_COL) {
        const double *c = d.colliders + 8 * tid;
        cols[tid] = Col{(int)c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7]};
        colf[tid][0] = (float)c[3];
        colf[tid][1] = (float)c[4];
    }

    for (int sc_seq = 0;; ++sc_seq) {
        if (!GR && tid == 0 && crank == 0) sc_next = atomicAdd(d.work, 1);
        int sc;
        if constexpr (GR) {  // the whole grid on each scene in turn
            sc = sc_seq;
        } else if constexpr (CL) {  // rank 0 takes the next scene; the cluster reads it from rank 0
            cg::cluster_group cl = cg::this_cluster();
            cluster_barrier();
            sc = *cl.map_shared_rank(&sc_next, 0);
            cluster_barrier();  // every read of rank 0's sc_next done before any block moves on or exits
        } else {
            block_barrier();
            sc = sc_next;
        }
        if (sc >= d.n_scenes) break;
        d2f_seg sg = d.segs[sc];
        if constexpr (!F_RARE) { sg.naff = 0; sg.naffn = 0; sg.nten = 0; sg.ntent = 0; sg.nsp = 0; sg.npe = 0; }
        if constexpr (!F_IPC) sg.ne = 0;
        const int n0 = sg.node0, n1 = sg.node0 + sg.nn;
        const int t0 = sg.tri0, t1 = sg.tri0 + sg.nt;
        const bool scene_ipc = has_ipc && sg.ne > 0;
        const bool scene_rig = sg.nrig > 0;
        const bool scene_rare = scene_ipc || sg.naff > 0 || sg.nten > 0 || sg.nsp > 0 || sg.npe > 0;  // terms with FP64 contributions
        const int nbl = sg.nb;
        if (tid < n_col && tid < MAX_COL) {
            colmu[tid] = d.col_mu_env ? d.col_mu_env[sc * n_col + tid] : cols[tid].mu;
            colmuf[tid] = (float)colmu[tid];
        }

        auto xpos = [&](int n) -> double2 {  // FP64 position x_b + (x - x_b)
            const double2 a = XBd[n];
            const float2 b = XR[n];
            return make_double2(a.x + (double)b.x, a.y + (double)b.y);
        };
        auto xbpos = [&](int n) -> double2 { return XBd[n]; };  // FP64 position at the base x_b

        // The base of the iteration: positions x = x_b + r with x_b in FP64 and the offset r in
        // FP32, and the gradient g = g0 + (g - g0) with g0 = elastic force + tendon force
        // - h^2 f_ext at x_b evaluated in FP64 and kept as a compensated FP32 pair, the
        // increment formed from r in FP32. Rebuilt at the step start and every REBASE
        // iterations (x_b += r, r = 0): the offsets and increments shrink as the solve
        // converges, so neither the positions' FP32 resolution nor the large, mutually
        // cancelling forces of a loaded body limit how far it converges (iterative refinement).
        auto build_base = [&]() {
            for (int i = n0 + gt; i < n1; i += GS) {
                const double2 b = XBd[i], xn = Xn[i];
                const float2 r = XR[i];
                const double2 xb = make_double2(b.x + (double)r.x, b.y + (double)r.y);
                XBd[i] = xb;
                XR[i] = make_float2(0.f, 0.f);
                const float2 db = make_float2((float)(xb.x - xn.x), (float)(xb.y - xn.y));
                DB[i] = db;
                XD[i] = db;
            }
            gsync();
            for (int t = t0 + gt; t < t1; t += GS) {
                const int i0 = d.tri[3 * t], i1 = d.tri[3 * t + 1], i2 = d.tri[3 * t + 2];
                const double2 a0 = XBd[i0], a1 = XBd[i1], a2 = XBd[i2], r1 = Dm2[2 * t], r2 = Dm2[2 * t + 1];
                const double e1x = (a1.x - a0.x) - r1.x, e1y = (a1.y - a0.y) - r1.y;
                const double e2x = (a2.x - a0.x) - r2.x, e2y = (a2.y - a0.y) - r2.y;
                DU0[t] = make_float4((float)e1x, (float)e1y, (float)e2x, (float)e2y);
                const float4 Bf = Bm[t];
                const double bx = Bf.x, by = Bf.y, bz = Bf.z, bw = Bf.w;
                const double H00 = e1x * bx + e2x * bz, H01 = e1x * by + e2x * bw;
                const double H10 = e1y * bx + e2y * bz, H11 = e1y * by + e2y * bw;
                const double dH = H00 * H11 - H01 * H10, Jm1 = (H00 + H11) + dH, J = 1.0 + Jm1;
                const double logJ = J > 1.0e-6 ? log1p(Jm1) : log(1.0e-6);
                const double iJ = J != 0.0 ? 1.0 / J : 0.0;
                const double mu = Mu[t], la = La[t], ll = la * logJ, onepJ = 1.0 + J;
                // cancellation-free first Piola stress of F = I + H
                const double P00 = mu * ((H00 * onepJ + dH) * iJ) + ll * ((1.0 + H11) * iJ);
                const double P01 = mu * ((J * H01 + H10) * iJ) + ll * (-H10 * iJ);
                const double P10 = mu * ((J * H10 + H01) * iJ) + ll * (-H01 * iJ);
                const double P11 = mu * ((H11 * onepJ + dH) * iJ) + ll * ((1.0 + H00) * iJ);
                const double hA = h2 * (double)Ar[t];
                const double g1x = hA * (P00 * bx + P01 * by), g1y = hA * (P10 * bx + P11 * by);
                const double g2x = hA * (P00 * bz + P01 * bw), g2y = hA * (P10 * bz + P11 * bw);
                Esc64[3 * t] = make_double2(-(g1x + g2x), -(g1y + g2y));
                Esc64[3 * t + 1] = make_double2(g1x, g1y);
                Esc64[3 * t + 2] = make_double2(g2x, g2y);
            }
            gsync();
            for (int i = n0 + gt; i < n1; i += GS) {
                double gx = 0.0, gy = 0.0;
                for (int k = __ldg(d.inc_ptr + i); k < __ldg(d.inc_ptr + i + 1); ++k) {
                    const double2 c = Esc64[__ldg(d.inc + k)];
                    gx += c.x; gy += c.y;
                }
                if (d.fext) {
                    const double2 f = Fx[i];
                    gx -= h2 * f.x; gy -= h2 * f.y;
                }
                G0d[i] = make_double2(gx, gy);
            }
            gsync();
            if (sg.nten > 0) {  // tendon force at x_b (Tendon.grad_diag, actuation.py:169-228)
                for (int k = sg.ten0 + gt; k < sg.ten0 + sg.nten; k += GS) {
                    double L = 0.0;
                    for (int j = sg.tent0; j < sg.tent0 + sg.ntent; ++j) {
                        if (d.t_tid[j] != k) continue;
                        const int m = d.t_nxt[j];
                        if (m < 0) continue;
                        const double2 xa = xbpos(d.t_node[j]), xb = xbpos(d.t_node[m]);
                        const double ex = xb.x - xa.x, ey = xb.y - xa.y;
                        L += sqrt(ex * ex + ey * ey);
                    }
                    double tau;
                    if (d.t_stiff[k] > 0.0) {
                        const double ext = L - d.t_L0[k];
                        tau = ext > 0.0 ? d.t_stiff[k] * ext : 0.0;
                    } else {
                        tau = dmax(d.t_Tcmd[k], 0.0);
                    }
                    d.t_state[4 * k + 1] = tau;  // tension at x_b, read by the increments
                }
                gsync();
                for (int j = sg.tent0 + gt; j < sg.tent0 + sg.ntent; j += GS) {
                    const int n = d.t_node[j];
                    const double tau = d.t_state[4 * d.t_tid[j] + 1];
                    const double2 g = tendon_dlen(xbpos, d.t_node, d.t_prv[j], d.t_nxt[j], n);
                    atomicAdd(&G0d[n].x, h2 * tau * g.x);
                    atomicAdd(&G0d[n].y, h2 * tau * g.y);
                }
                gsync();
            }
            if (sg.nsp > 0 || sg.npe > 0) {  // spring and pressure forces at x_b (FP64)
                for (int k = sg.sp0 + gt; k < sg.sp0 + sg.nsp; k += GS) {
                    const int a = d.sp_a[k], b = d.sp_b[k];
                    const SpringAt sa = spring_at(XBd[a], b >= 0 ? XBd[b] : spring_anchor(d, k), d.sp_k[k], d.sp_L0[k]);
                    const double gx = h2 * sa.ten * sa.nx, gy = h2 * sa.ten * sa.ny;
                    atomicAdd(&G0d[a].x, gx); atomicAdd(&G0d[a].y, gy);
                    if (b >= 0) { atomicAdd(&G0d[b].x, -gx); atomicAdd(&G0d[b].y, -gy); }
                }
                for (int e = sg.pe0 + gt; e < sg.pe0 + sg.npe; e += GS) {
                    const int a = d.pe_a[e], b = d.pe_b[e];
                    const double2 xa = XBd[a], xb = XBd[b];
                    const double sp = -0.5 * h2 * d.ch_p[d.pe_ch[e]];
                    const double gx = sp * (xb.y - xa.y), gy = -sp * (xb.x - xa.x);
                    atomicAdd(&G0d[a].x, gx); atomicAdd(&G0d[a].y, gy);
                    atomicAdd(&G0d[b].x, gx); atomicAdd(&G0d[b].y, gy);
                }
                gsync();
            }
            for (int i = n0 + gt; i < n1; i += GS) {  // to a compensated FP32 pair, in place
                const double2 g = G0d[i];
                const float hx = (float)g.x, hy = (float)g.y;
                G0[i] = make_float4(hx, hy, (float)(g.x - (double)hx), (float)(g.y - (double)hy));
            }
            gsync();
        };

        // ================================================================ step setup (FP64, once per step)
        for (int i = n0 + gt; i < n1; i += GS) {
            const double2 xi = X[i], vi = Vv[i];
            Xn[i] = xi;
            XD[i] = make_float2(0.f, 0.f);
            XBd[i] = xi;
            XR[i] = make_float2(0.f, 0.f);
            GD[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            HVM[i] = make_float4((float)(dt * d.drag * vi.x), (float)(dt * d.drag * vi.y), (float)d.mass[i], 0.f);
            {  // packed static node info: bits 0-1 free mask, 2 affine, 3 rigid, 4-7 rigid piece (15: look up)
                int f = d.free_mask[i];
                if (d.node_aff[i] >= 0) f |= NI_AFF;
                const int kr = d.node_rig[i];
                if (kr >= 0) {
                    const int lb = d.r_grp[kr] - sg.rig0;
                    f |= NI_RIG | ((lb < 15 ? lb : 15) << 4);
                }
                NINFO[i] = make_int2(f, d.node_bslot[i]);
            }
            G[i] = make_float2(0.f, 0.f);
            P[i] = make_float2(0.f, 0.f);
        }
        if (tid == 0) {
            S.active = 1; S.iters = 0; S.dE0 = 0.0; S.status = 0; S.pending = 0;
            S.alpha = d.alpha_max; S.pHp = 0.0; S.q_inf = 0.0; S.alpha_s = 1.0;
            S.ncand = 0; S.rebuild = 1; S.gn0 = 0.0; S.beta = 0.0;
            S.motion = 0.0; S.csx = 0.0; S.csy = 0.0;
            F.alpha = falpha_max; F.beta = 0.f; F.pinf = 0.f; F.gn0 = 0.f; F.gn2 = 0.f;
            F.gPg = 0.f; F.g_Py = 0.f; F.y_Py = 0.f; F.csx = 0.f; F.csy = 0.f; F.mpx = 0.f; F.mpy = 0.f; F.inv_m = 0.f;
        }
        gsync();
        for (int j = gt; j < nbl; j += GS) {  // half-space distances at x_n
            const double2 xb = Xn[d.bnd[sg.bnd0 + j]];
            for (int k = 0; k < n_col; ++k) {
                const Col c = cols[k];
                if (c.kind == 4) PHI0[(size_t)d.bnd[sg.bnd0 + j] * n_col + k] = (float)(c.rx * (xb.x - c.cx) + c.ry * (xb.y - c.cy));
            }
        }
        if (!scene_ipc) {  // apply_bc_kernel, kernels.py:53-59: x = target
            for (int b = sg.bc0 + gt; b < sg.bc0 + sg.nbc; b += GS) {
                const int n = d.bc_idx[b];
                const double2 tg = Tgt[b], xn = Xn[n];
                XD[n] = make_float2((float)(tg.x - xn.x), (float)(tg.y - xn.y));
                XBd[n] = tg;
            }
        }
        // rigid pieces: step-start centroid c_n (FP64) and the arms x_n - c_n (FP32)
        for (int b = sg.rig0; b < sg.rig0 + sg.nrig; ++b) {
            double c[3] = {0.0, 0.0, 0.0};
            for (int k = sg.rign0 + gt; k < sg.rign0 + sg.nrign; k += GS) {
                if (d.r_grp[k] != b) continue;
                const int i = d.r_node[k];
                const double m = d.mass[i];
                const double2 xi = Xn[i];
                c[0] += m * xi.x; c[1] += m * xi.y; c[2] += m;
            }
            const int ops3[3] = {0, 0, 0};
            scene_reduce<NT, CS, 3>(c, ops3, red, cres, gxp);
            const double cx = c[0] / c[2], cy = c[1] / c[2];
            for (int k = sg.rign0 + gt; k < sg.rign0 + sg.nrign; k += GS) {
                if (d.r_grp[k] != b) continue;
                const int i = d.r_node[k];
                const double2 xi = Xn[i];
                RARM[i] = make_float2((float)(xi.x - cx), (float)(xi.y - cy));
            }
            if (tid == 0 && crank == 0) { d.r_acc[3 * b] = cx; d.r_acc[3 * b + 1] = cy; d.r_acc[3 * b + 2] = c[2]; }
            if (tid == 0 && sg.nrig == 1) F.inv_m = (float)(1.0 / c[2]);
        }
        gsync();

        build_base();

        // ---------------------------------------------------------------- contact candidates
        // As in the FP64 kernel, but the list is rebuilt at every step start (x_n changed) and
        // its validity inside a step is the FP32 motion dx - dx_ref of the boundary nodes.
        // true while every candidate pair is provably out of reach: its distance at the list
        // build (dmin_c, conservative) minus twice the largest node move since then; the pair
        // passes and the ACCD replay would find nothing and are skipped (same result)
        bool ipc_far = false;
        auto ipc_refresh = [&]() {
            // rebuild when the nodes may have moved skin/2 since the last build: every node
            // moves at most alpha |p|_inf per iteration (alpha_s q_inf per sweep), summed in
            // S.motion — a bound, so no reduction over the nodes is needed
            if (!(S.rebuild || 2.0 * S.motion >= d.skin)) {
                ipc_far = S.dmin_c - 2.0 * S.motion >= d.reach;
                return;
            }
            gsync();
            // boundary positions in FP32 relative to the first boundary node: in shared memory
            // (every block its own copy), or for hashed scenes in PB, written once per scene
            // (the hashed build is compiled into the cluster kernels only: the batch kernel, a
            // block per scene of small scenes, keeps its registers for the iteration)
            const bool hashed = CL && nbl >= HASH_MIN_NB;
            float2 *P32 = hashed ? PB + sg.bnd0 : pos32;
            const double2 anchor = xpos(d.bnd[sg.bnd0]);
            for (int j = hashed ? gt : tid; j < nbl; j += hashed ? GS : NT) {
                const double2 xb = xpos(d.bnd[sg.bnd0 + j]);
                P32[j] = make_float2((float)(xb.x - anchor.x), (float)(xb.y - anchor.y));
            }
            if (hashed) gsync();
            const float rad = (float)(d.reach + d.skin);
            const float slack = 1.0e-5f * rad;
            float dmn = 3.0e38f;
            // edge k, slot j: a candidate when within reach + skin and not excluded
            auto pair_keep = [&](int k, int j, float &dd) -> bool {
                const int ge = sg.edge0 + k;
                const int a = d.ea[ge], b = d.eb[ge];
                const int pn = d.bnd[sg.bnd0 + j];
                if (pn == a || pn == b) return false;
                const int la = d.node_bslot[a] - sg.bnd0, lb = d.node_bslot[b] - sg.bnd0;
                const float2 pa = P32[la], pb = P32[lb], pp = P32[j];
                const float abx = pb.x - pa.x, aby = pb.y - pa.y;
                const float wx = pp.x - pa.x, wy = pp.y - pa.y;
                float t = (wx * abx + wy * aby) / fmaxf(abx * abx + aby * aby, 1e-30f);
                t = fminf(fmaxf(t, 0.f), 1.f);
                const float dx = wx - t * abx, dy = wy - t * aby;
                dd = sqrtf(dx * dx + dy * dy);
                return dd <= rad + slack && !excluded(d, sg.bnd0 + j, d.ela[ge]) && !excluded(d, sg.bnd0 + j, d.elb[ge]);
            };
            int base_off = 0, n_all = 0;
            // the blocks of a cluster: their kept-pair counts, then each block's offset (the
            // lower ranks' pairs) and the scene's total; the list comes out in pair order
            auto cluster_offsets = [&](int mine) {
                if constexpr (CL) {
                    if (tid == 0) s_cnt = 0;
                    block_barrier();
                    if ((tid & 31) == 0 && mine) atomicAdd(&s_cnt, mine);
                    if constexpr (GR) {  // the counts through global memory
                        block_barrier();
                        if (tid == 0) gxv.cnt[crank] = s_cnt;
                        grid_barrier(gxv);
                        for (int r = 0; r < NBS; ++r) {
                            const int c = *reinterpret_cast<volatile int *>(gxv.cnt + r);
                            if (r < crank) base_off += c;
                            n_all += c;
                        }
                        grid_barrier(gxv);  // every read done before the counts are reused
                    } else {
                        cg::cluster_group cl = cg::this_cluster();
                        cluster_barrier();
                        for (int r = 0; r < CS; ++r) {
                            const int c = *cl.map_shared_rank(&s_cnt, r);
                            if (r < crank) base_off += c;
                            n_all += c;
                        }
                        cluster_barrier();
                    }
                }
            };
            if (hashed) {
                // counting sort of the slots by the hash of their cell (cells of rad + 2 slack),
                // every block its own table in shared memory: bucket ends, then the slots
                unsigned *hend = reinterpret_cast<unsigned *>(pos32);
                int *hslot = reinterpret_cast<int *>(pos32) + HASH_B;
                const float R = rad + 2.0f * slack, icell = 1.0f / R;
                auto cell_of = [&](float v) -> int { return (int)floorf(v * icell); };
                auto bucket = [&](int cx, int cy) -> int {
                    return (int)(((unsigned)cx * 73856093u ^ (unsigned)cy * 19349663u) & (unsigned)(HASH_B - 1));
                };
                for (int h = tid; h < HASH_B; h += NT) hend[h] = 0u;
                block_barrier();
                for (int j = tid; j < nbl; j += NT) {
                    const float2 p = P32[j];
                    atomicAdd(&hend[bucket(cell_of(p.x), cell_of(p.y))], 1u);
                }
                block_barrier();
                {  // exclusive scan of the counts: NT consecutive buckets per pass
                    unsigned carry = 0;
                    for (int base = 0; base < HASH_B; base += NT) {
                        const int h = base + tid;
                        const unsigned c = h < HASH_B ? hend[h] : 0u;
                        unsigned incl = c;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
                            if ((tid & 31) >= o) incl += u;
                        }
                        if ((tid & 31) == 31) s_wcnt[tid >> 5] = (int)incl;
                        block_barrier();
                        unsigned before = carry, tot = 0;
                        for (int w = 0; w < NW; ++w) {
                            if (w < (tid >> 5)) before += (unsigned)s_wcnt[w];
                            tot += (unsigned)s_wcnt[w];
                        }
                        if (h < HASH_B) hend[h] = before + incl - c;  // the bucket's start
                        carry += tot;
                        block_barrier();
                    }
                }
                for (int j = tid; j < nbl; j += NT) {  // the starts advance to the ends
                    const float2 p = P32[j];
                    hslot[atomicAdd(&hend[bucket(cell_of(p.x), cell_of(p.y))], 1u)] = j;
                }
                block_barrier();
                // edge k's candidates: the slots in the buckets of the cells its box (grown by
                // R) covers, each bucket once; all slots for an edge longer than that allows
                auto walk = [&](int k, bool wr, int off) -> int {
                    const int ge = sg.edge0 + k;
                    const float2 pa = P32[d.node_bslot[d.ea[ge]] - sg.bnd0], pb = P32[d.node_bslot[d.eb[ge]] - sg.bnd0];
                    const int cx0 = cell_of(fminf(pa.x, pb.x) - R), cx1 = cell_of(fmaxf(pa.x, pb.x) + R);
                    const int cy0 = cell_of(fminf(pa.y, pb.y) - R), cy1 = cell_of(fmaxf(pa.y, pb.y) + R);
                    int n = 0;
                    auto take = [&](int j) {
                        float dd;
                        if (!pair_keep(k, j, dd)) return;
                        dmn = fminf(dmn, dd);
                        if (wr && off + n < sg.ncap) d.cand[sg.cand0 + off + n] = (int)(((unsigned)k << 16) | (unsigned)j);
                        ++n;
                    };
                    // (non-finite positions give saturated cells: a huge box, so every slot)
                    const long ncell = ((long)cx1 - (long)cx0 + 1) * ((long)cy1 - (long)cy0 + 1);
                    if (cx1 < cx0 || cy1 < cy0 || ncell > 16) {
                        for (int j = 0; j < nbl; ++j) take(j);
                        return n;
                    }
                    for (int cy = cy0; cy <= cy1; ++cy) {
                        for (int cx = cx0; cx <= cx1; ++cx) {
                            const int h = bucket(cx, cy);
                            bool seen = false;  // the same bucket from an earlier cell of this box
                            for (int cy2 = cy0; cy2 <= cy && !seen; ++cy2)
                                for (int cx2 = cx0; cx2 <= cx1; ++cx2) {
                                    if (cy2 == cy && cx2 >= cx) break;
                                    if (bucket(cx2, cy2) == h) { seen = true; break; }
                                }
                            if (seen) continue;
                            const int s1 = (int)hend[h], s0 = h > 0 ? (int)hend[h - 1] : 0;
                            for (int q = s0; q < s1; ++q) take(hslot[q]);
                        }
                    }
                    return n;
                };
                // this block's contiguous share of the edges (all of them for a block per scene)
                const int echunk = (sg.ne + NBS - 1) / NBS;
                const int e0 = CL ? min(crank * echunk, sg.ne) : 0;
                const int e1 = CL ? min(e0 + echunk, sg.ne) : sg.ne;
                if constexpr (CL) {  // pass 1: count
                    int mine = 0;
                    for (int k = e0 + tid; k < e1; k += NT) mine += walk(k, false, 0);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
                    cluster_offsets(mine);
                }
                if (tid == 0) S.count = base_off;
                block_barrier();
                for (int base = e0; base < e1; base += NT) {  // pass 2: count, place, write
                    const int k = base + tid;
                    const int c = k < e1 ? walk(k, false, 0) : 0;
                    int incl = c;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int u = __shfl_up_sync(0xffffffffu, incl, o);
                        if ((tid & 31) >= o) incl += u;
                    }
                    if ((tid & 31) == 31) s_wcnt[tid >> 5] = incl;
                    block_barrier();
                    int off = S.count + incl - c, tot = 0;
                    for (int w = 0; w < NW; ++w) {
                        if (w < (tid >> 5)) off += s_wcnt[w];
                        tot += s_wcnt[w];
                    }
                    if (c > 0) walk(k, true, off);
                    block_barrier();
                    if (tid == 0) S.count += tot;
                }
            } else {
                const long npair = (long)sg.ne * nbl;
                // this block's contiguous share of the pair space (all of it for a block per scene)
                const long chunk = (npair + NBS - 1) / NBS;
                const long q0 = CL ? (crank * chunk < npair ? crank * chunk : npair) : 0;
                const long q1 = CL ? (q0 + chunk < npair ? q0 + chunk : npair) : npair;
                block_barrier();  // pos32 complete
                if constexpr (CL) {  // pass 1: count
                    int mine = 0;
                    for (long base = q0; base < q1; base += NT) {
                        const long q = base + tid;
                        float dd;
                        const bool keep = q < q1 && pair_keep((int)(q / nbl), (int)(q % nbl), dd);
                        mine += __popc(__ballot_sync(0xffffffffu, keep));
                    }
                    cluster_offsets((tid & 31) == 0 ? mine : 0);
                }
                if (tid == 0) S.count = base_off;
                block_barrier();
                for (long base = q0; base < q1; base += NT) {
                    const long q = base + tid;
                    bool keep = false;
                    int k = 0, j = 0;
                    if (q < q1) {
                        k = (int)(q / nbl);
                        j = (int)(q - (long)k * nbl);
                        float dd;
                        keep = pair_keep(k, j, dd);
                        if (keep) dmn = fminf(dmn, dd);
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, keep);
                    const int lane = tid & 31, warp = tid >> 5;
                    if (lane == 0) s_wcnt[warp] = __popc(bal);
                    block_barrier();
                    int off = S.count + __popc(bal & ((1u << lane) - 1u)), tot = 0;
                    for (int w = 0; w < NW; ++w) {
                        if (w < warp) off += s_wcnt[w];
                        tot += s_wcnt[w];
                    }
                    if (keep && off < sg.ncap) d.cand[sg.cand0 + off] = (int)(((unsigned)k << 16) | (unsigned)j);
                    block_barrier();
                    if (tid == 0) S.count += tot;
                }
            }
            block_barrier();
            double vm[1] = {(double)dmn};
            const int opm[1] = {2};
            scene_reduce<NT, CS, 1>(vm, opm, red, cres, gxp);
            if (tid == 0) {
                const int cnt = CL ? n_all : S.count;
                if (cnt > sg.ncap) { S.status = D2F_ECAP; S.ncand = sg.ncap; }
                else S.ncand = cnt;
                S.rebuild = 0;
                S.motion = 0.0;
                S.dmin_c = vm[0] - 1.0e-4 * (double)rad;  // FP32 rounding of the build distances
            }
            gsync();
            ipc_far = S.dmin_c >= d.reach;
        };

        auto kin_dir = [&](int n) -> double2 {
            const int b = d.node_bc[n];
            if (b < 0) return make_double2(0.0, 0.0);
            const double2 t = Tgt[b], x = xpos(n);
            return make_double2(t.x - x.x, t.y - x.y);
        };
        // One candidate pair in FP64 at x_b + r (ipc_pair_kernel + _pair, ipc_contact.py:130-296);
        // mode 0: gradient and diagonal, 1: curvature along p and the ACCD profile, 2: energy,
        // 3: the kinematic sweep's ACCD profile
        auto pair64 = [&](int c, int mode, double &acc_pHp, double t_c) {
            const double idhat = d.ipc_dhat, ikappa = d.ipc_kappa, reach = d.reach, gap = d.gap;
            const double dlo = 1.0e-9 * idhat, onset = 0.02 * idhat;
            const double mu_s = d.friction ? d.ipc_mu : 0.0;
            const int per_body = d.friction ? d.per_body : 0;
            const double floor_ = d.bc_floor * idhat;
            const unsigned packed = (unsigned)d.cand[sg.cand0 + c];
            const int k = (int)(packed >> 16), j = (int)(packed & 0xffffu);
            const int ge = sg.edge0 + k;
            const int a = d.ea[ge], b = d.eb[ge], pn = d.bnd[sg.bnd0 + j];
            const double2 xa = xpos(a), xb = xpos(b), xp = xpos(pn);
            const double abx = xb.x - xa.x, aby = xb.y - xa.y;
            const double L2 = dmax(abx * abx + aby * aby, 1.0e-30), Ll = sqrt(L2);
            const double wx = xp.x - xa.x, wy = xp.y - xa.y;
            const double tt = (wx * abx + wy * aby) / L2;
            double dvx = wx - tt * abx, dvy = wy - tt * aby;
            if (tt <= 0.0) { dvx = wx; dvy = wy; }
            else if (tt >= 1.0) { dvx = xp.x - xb.x; dvy = xp.y - xb.y; }
            const double dd = sqrt(dvx * dvx + dvy * dvy);
            if (!(dd < reach)) {
                if (mode == 1 || mode == 3) Ctr[sg.cand0 + c] = make_double2(1.0e300, 1.0e300);
                return;
            }
            if (mode == 1 || mode == 3) {
                double keep = dmax(gap * dd, idhat - onset);
                if (dd < idhat) keep = dd - dmin(2.0 * (idhat - dd) + onset, 0.5 * dd);
                if (mode == 3) keep = dmin(dd, dmax(gap * dd, floor_));
                double2 qp, qa, qb;
                if (mode == 3) { qp = kin_dir(pn); qa = kin_dir(a); qb = kin_dir(b); }
                else {
                    const float2 u0 = P[pn], u1 = P[a], u2 = P[b];
                    qp = make_double2(u0.x, u0.y); qa = make_double2(u1.x, u1.y); qb = make_double2(u2.x, u2.y);
                }
                double T;
                const double Rv = accd_profile(xp.x, xp.y, xa.x, xa.y, xb.x, xb.y, qp.x, qp.y, qa.x, qa.y,
                                               qb.x, qb.y, keep, t_c, T);
                Ctr[sg.cand0 + c] = make_double2(T, Rv);
            }
            if (mode == 3) return;
            double mu_p = mu_s;
            if (per_body) {
                const double mi = d.mu_node[pn], mj = d.mu_node[a], sm = mi + mj;
                mu_p = sm > 0.0 ? 2.0 * mi * mj / sm : 0.0;
            }
            auto term = [&](double coef, int ip, int ia, int ib, double wa, double wb, double dist, double nx,
                            double ny, double ddd) {
                const double bp = barrier_bp<double>(dist, idhat);
                const double f_n = -ikappa * bp;
                const double tnx = -ny, tny = nx;
                const float2 di = XD[ip], da = XD[ia], db = XD[ib];  // slip since the step began
                const double ux = (double)di.x - wa * (double)da.x - wb * (double)db.x;
                const double uy = (double)di.y - wa * (double)da.y - wb * (double)db.y;
                const double ut = ux * tnx + uy * tny;
                const double vt = dabs(ut) * inv_dt;
                const double kt = mu_p * f_n * inv_dt / dmax(vt, d.epsv);
                if (mode == 0) {
                    const double bpp = barrier_bpp<double>(dist, idhat);
                    const double s = mu_p * f_n * (ut * inv_dt / dmax(vt, d.epsv));
                    const double gx = h2 * (-f_n * nx + s * tnx), gy = h2 * (-f_n * ny + s * tny);
                    const double hx = h2 * (ikappa * bpp * nx * nx + kt * tnx * tnx);
                    const double hy = h2 * (ikappa * bpp * ny * ny + kt * tny * tny);
                    const int ids[3] = {ip, ia, ib};
                    const double cg[3] = {coef, -coef * wa, -coef * wb};
                    const double ch[3] = {coef, coef * wa * wa, coef * wb * wb};
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const int n = ids[q];
                        const uint8_t fm = d.free_mask[n];
                        float *gp_ = reinterpret_cast<float *>(G + n);
                        float *dp_ = reinterpret_cast<float *>(D + n);
                        if (fm & 1) atomicAdd(gp_, (float)(cg[q] * gx));
                        if (fm & 2) atomicAdd(gp_ + 1, (float)(cg[q] * gy));
                        atomicAdd(dp_, (float)(ch[q] * hx));
                        atomicAdd(dp_ + 1, (float)(ch[q] * hy));
                    }
                } else if (mode == 2) {  // energy: barrier + lagged friction (ipc_contact.py:414-429)
                    const double asl = d.epsv / inv_dt, au = dabs(ut);
                    const double f0 = au < asl ? au * au / (2.0 * asl) : au - 0.5 * asl;
                    acc_pHp += coef * h2 * (ikappa * barrier_b<double>(dist, idhat) + mu_p * f_n * f0);
                } else {
                    const double bpp = barrier_bpp<double>(dist, idhat);
                    const float2 u0 = P[ip], u1 = P[ia], u2 = P[ib];
                    const double qx = (double)u0.x - wa * (double)u1.x - wb * (double)u2.x;
                    const double qy = (double)u0.y - wa * (double)u1.y - wb * (double)u2.y;
                    const double dn = qx * nx + qy * ny, dt_ = qx * tnx + qy * tny;
                    const double val = dmax(ikappa * (bpp * dn * dn + bp * ddd), 0.0);
                    acc_pHp += coef * h2 * (val + kt * dt_ * dt_);
                }
            };
            if (tt > 0.0 && tt < 1.0 && dd < idhat) {
                const double dist = dmax(dd, dlo);
                double ddd = 0.0;
                if (mode == 1) {
                    const float2 pb_ = P[b], pa_ = P[a], pp_ = P[pn];
                    const double dex = (double)pb_.x - (double)pa_.x, dey = (double)pb_.y - (double)pa_.y;
                    const double dwx = (double)pp_.x - (double)pa_.x, dwy = (double)pp_.y - (double)pa_.y;
                    const double c0 = abx * wy - aby * wx;
                    const double c1 = (dex * wy - dey * wx) + (abx * dwy - aby * dwx);
                    const double c2 = 2.0 * (dex * dwy - dey * dwx);
                    const double L1 = (abx * dex + aby * dey) / Ll;
                    const double Lq = ((dex * dex + dey * dey) - L1 * L1) / Ll;
                    const double s0 = c0 / Ll;
                    const double s1 = (c1 - s0 * L1) / Ll;
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
                const double nx = wx / d_a, ny = wy / d_a;
                double ddd = 0.0;
                if (mode == 1) {
                    const float2 pp_ = P[pn], pa_ = P[a];
                    const double dwx = (double)pp_.x - (double)pa_.x, dwy = (double)pp_.y - (double)pa_.y;
                    const double dn = dwx * nx + dwy * ny;
                    ddd = ((dwx * dwx + dwy * dwy) - dn * dn) / d_a;
                }
                term(coef_a, pn, a, b, 1.0, 0.0, d_a, nx, ny, ddd);
            }
            double coef_b = -d.cb[ge];
            if (tt >= 1.0) coef_b += 1.0;
            const double wbx = xp.x - xb.x, wby = xp.y - xb.y;
            double d_b = sqrt(wbx * wbx + wby * wby);
            if (coef_b != 0.0 && d_b < idhat) {
                d_b = dmax(d_b, dlo);
                const double nx = wbx / d_b, ny = wby / d_b;
                double ddd = 0.0;
                if (mode == 1) {
                    const float2 pp_ = P[pn], pb_ = P[b];
                    const double dwx = (double)pp_.x - (double)pb_.x, dwy = (double)pp_.y - (double)pb_.y;
                    const double dn = dwx * nx + dwy * ny;
                    ddd = ((dwx * dwx + dwy * dwy) - dn * dn) / d_b;
                }
                term(coef_b, pn, a, b, 0.0, 1.0, d_b, nx, ny, ddd);
            }
        };
        auto ipc_pairs = [&](int mode, double &acc_pHp, double t_c) {
            if (ipc_far) return;  // every pair out of reach: no term, no cap
            const int nc = S.ncand;
            for (int c = gt; c < nc; c += GS) pair64(c, mode, acc_pHp, t_c);
        };
        // Modes 0 and 1 of the pair pass in FP32: the barrier and friction arithmetic and the
        // ACCD profile on the pair's geometry taken relative to node a — the FP64 differences of
        // the base positions, rounded once, plus the FP32 offsets — which resolves the pair's own
        // magnitudes (~d-hat) to ~1e-7 of them. A pair with a term closer than 1e-3 d-hat, where
        // the barrier nears its singularity, takes the FP64 pass (pair64). Mode 1's curvature
        // goes to the compensated pair accf, the FP64 fallback's to acc64.
        auto ipc_pairs32 = [&](int mode, FF &accf, double &acc64, float t_c) {
            if (ipc_far) return;  // every pair out of reach: no term, no cap
            const float idhat = (float)d.ipc_dhat, ikappa = (float)d.ipc_kappa, reach = (float)d.reach;
            const float gap = (float)d.gap, dlo = 1.0e-9f * idhat, onset = 0.02f * idhat, dnear = 1.0e-3f * idhat;
            const float mu_s = d.friction ? (float)d.ipc_mu : 0.f;
            const int per_body = d.friction ? d.per_body : 0;
            const int nc = S.ncand;
            for (int c = gt; c < nc; c += GS) {
                const unsigned packed = (unsigned)d.cand[sg.cand0 + c];
                const int k = (int)(packed >> 16), j = (int)(packed & 0xffffu);
                const int ge = sg.edge0 + k;
                const int a = d.ea[ge], b = d.eb[ge], pn = d.bnd[sg.bnd0 + j];
                const double2 ba = XBd[a], bb = XBd[b], bp = XBd[pn];
                const float2 ra = XR[a], rb = XR[b], rp = XR[pn];
                // base differences in FP64, rounded once; offsets since the base in FP32
                const double abxb = bb.x - ba.x, abyb = bb.y - ba.y, wxb = bp.x - ba.x, wyb = bp.y - ba.y;
                const float fabx = (float)abxb, faby = (float)abyb, fwx = (float)wxb, fwy = (float)wyb;
                const float dabx = rb.x - ra.x, daby = rb.y - ra.y, dwx0 = rp.x - ra.x, dwy0 = rp.y - ra.y;
                const float abx = fabx + dabx, aby = faby + daby;
                const float wx = fwx + dwx0, wy = fwy + dwy0;
                const float wbx = (float)(bp.x - bb.x) + (rp.x - rb.x), wby = (float)(bp.y - bb.y) + (rp.y - rb.y);
                // cross(ab, w) = |ab| x the signed distance of p from the edge's line: the base
                // product in FP64 and the increment in FP32, so the distance of a close pair keeps
                // FP32's relative accuracy (w - t ab in FP32 would lose it to cancellation, by the
                // ratio of the edge length to the distance)
                const float cr = (float)(abxb * wyb - abyb * wxb) +
                                 (((fabx * dwy0 - faby * dwx0) + (dabx * fwy - daby * fwx)) + (dabx * dwy0 - daby * dwx0));
                const float L2 = fmaxf(abx * abx + aby * aby, 1.0e-30f), Ll = sqrtf(L2);
                const float tt = (wx * abx + wy * aby) / L2;
                float dd;
                if (tt <= 0.f) dd = sqrtf(wx * wx + wy * wy);
                else if (tt >= 1.f) dd = sqrtf(wbx * wbx + wby * wby);
                else dd = fabsf(cr) / Ll;
                if (!(dd < reach)) {
                    if (mode == 1) Ctr[sg.cand0 + c] = make_double2(1.0e300, 1.0e300);
                    continue;
                }
                const float d_a = sqrtf(wx * wx + wy * wy), d_b = sqrtf(wbx * wbx + wby * wby);
                if (fminf(dd, fminf(d_a, d_b)) < dnear) {  // near the barrier's singularity: FP64
                    pair64(c, mode, acc64, (double)t_c);
                    continue;
                }
                const float2 pp_ = P[pn], pa_ = P[a], pb_ = P[b];
                if (mode == 1) {  // ACCD profile (ipc_contact.py:94-127), the FP64 pass's margins
                    float keep = fmaxf(gap * dd, idhat - onset);
                    if (dd < idhat) keep = dd - fminf(2.f * (idhat - dd) + onset, 0.5f * dd);
                    float T;
                    const float Rv = accd_profile_f(wx, wy, 0.f, 0.f, abx, aby, pp_.x, pp_.y, pa_.x, pa_.y, pb_.x, pb_.y,
                                                    keep, t_c, T);
                    Ctr[sg.cand0 + c] = make_double2(T >= 3.0e38f ? 1.0e300 : (double)T, (double)Rv);
                }
                float mu_p = mu_s;
                if (per_body) {
                    const float mi = (float)d.mu_node[pn], mj = (float)d.mu_node[a], sm = mi + mj;
                    mu_p = sm > 0.f ? 2.f * mi * mj / sm : 0.f;
                }
                auto term = [&](float coef, int ia, int ib, float wa, float wb, float dist, float nx, float ny, float ddd) {
                    const float bp1 = barrier_bp<float>(dist, idhat), bpp = barrier_bpp<float>(dist, idhat);
                    const float f_n = -ikappa * bp1;
                    const float tnx = -ny, tny = nx;
                    const float2 di = XD[pn], da = XD[ia], db = XD[ib];  // slip since the step began
                    const float ux = di.x - wa * da.x - wb * db.x, uy = di.y - wa * da.y - wb * db.y;
                    const float ut = ux * tnx + uy * tny;
                    const float vt = fabsf(ut) * finv_dt;
                    const float kt = mu_p * f_n * finv_dt / fmaxf(vt, fepsv);
                    if (mode == 0) {
                        const float sf = mu_p * f_n * (ut * finv_dt / fmaxf(vt, fepsv));
                        const float gx = fh2 * (-f_n * nx + sf * tnx), gy = fh2 * (-f_n * ny + sf * tny);
                        const float hx = fh2 * (ikappa * bpp * nx * nx + kt * tnx * tnx);
                        const float hy = fh2 * (ikappa * bpp * ny * ny + kt * tny * tny);
                        const int ids[3] = {pn, ia, ib};
                        const float cg[3] = {coef, -coef * wa, -coef * wb};
                        const float ch[3] = {coef, coef * wa * wa, coef * wb * wb};
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const int n = ids[q];
                            const uint8_t fm = d.free_mask[n];
                            float *gp_ = reinterpret_cast<float *>(G + n);
                            float *dp_ = reinterpret_cast<float *>(D + n);
                            if (fm & 1) atomicAdd(gp_, cg[q] * gx);
                            if (fm & 2) atomicAdd(gp_ + 1, cg[q] * gy);
                            atomicAdd(dp_, ch[q] * hx);
                            atomicAdd(dp_ + 1, ch[q] * hy);
                        }
                    } else {
                        const float2 u1 = P[ia], u2 = P[ib];
                        const float qx = pp_.x - wa * u1.x - wb * u2.x, qy = pp_.y - wa * u1.y - wb * u2.y;
                        const float dn = qx * nx + qy * ny, dt_ = qx * tnx + qy * tny;
                        const float val = fmaxf(ikappa * (bpp * dn * dn + bp1 * ddd), 0.f);
                        ff_add(accf, coef * fh2 * (val + kt * dt_ * dt_));
                    }
                };
                if (tt > 0.f && tt < 1.f && dd < idhat) {
                    const float dist = fmaxf(dd, dlo);
                    float ddd = 0.f;
                    if (mode == 1) {
                        const float dex = pb_.x - pa_.x, dey = pb_.y - pa_.y;
                        const float dwx = pp_.x - pa_.x, dwy = pp_.y - pa_.y;
                        const float c0 = cr;
                        const float c1 = (dex * wy - dey * wx) + (abx * dwy - aby * dwx);
                        const float c2 = 2.f * (dex * dwy - dey * dwx);
                        const float L1 = (abx * dex + aby * dey) / Ll;
                        const float Lq = ((dex * dex + dey * dey) - L1 * L1) / Ll;
                        const float s0 = c0 / Ll, s1 = (c1 - s0 * L1) / Ll;
                        ddd = (c2 - 2.f * s1 * L1 - s0 * Lq) / Ll;
                        if (c0 < 0.f) ddd = -ddd;
                    }
                    // the normal from the edge to the point: the edge's perpendicular on the point's side
                    const float sgn = cr >= 0.f ? 1.f / Ll : -1.f / Ll;
                    term(1.f, a, b, 1.f - tt, tt, dist, -aby * sgn, abx * sgn, ddd);
                }
                float coef_a = -(float)d.ca[ge];
                if (tt <= 0.f) coef_a += 1.f;
                if (coef_a != 0.f && d_a < idhat) {
                    const float dist = fmaxf(d_a, dlo), nx = wx / dist, ny = wy / dist;
                    float ddd = 0.f;
                    if (mode == 1) {
                        const float dwx = pp_.x - pa_.x, dwy = pp_.y - pa_.y, dn = dwx * nx + dwy * ny;
                        ddd = ((dwx * dwx + dwy * dwy) - dn * dn) / dist;
                    }
                    term(coef_a, a, b, 1.f, 0.f, dist, nx, ny, ddd);
                }
                float coef_b = -(float)d.cb[ge];
                if (tt >= 1.f) coef_b += 1.f;
                if (coef_b != 0.f && d_b < idhat) {
                    const float dist = fmaxf(d_b, dlo), nx = wbx / dist, ny = wby / dist;
                    float ddd = 0.f;
                    if (mode == 1) {
                        const float dwx = pp_.x - pb_.x, dwy = pp_.y - pb_.y, dn = dwx * nx + dwy * ny;
                        ddd = ((dwx * dwx + dwy * dwy) - dn * dn) / dist;
                    }
                    term(coef_b, a, b, 0.f, 1.f, dist, nx, ny, ddd);
                }
            }
        };
        auto tc_scan = [&](double m0) -> double {  // every thread calls; the result is thread 0's
            if (ipc_far) return m0;  // no pair in reach: every profile is (inf, inf)
            // A pair whose profile threshold T is >= m0 leaves the running minimum untouched at
            // any cap <= m0 (accd_profile: accd(m) = m for m <= T), so only the pairs with
            // T < m0 are replayed — found by warp ballots in candidate order, walked in that
            // order by thread 0 with the same per-edge reset: the result equals the full serial
            // replay.
            const int nc = S.ncand;
            if constexpr (CL) {
                // each block filters its contiguous share of the candidates into an ordered list
                // in shared memory; thread 0 of every block walks the lists in rank order
                // (distributed shared memory): the same pairs in the same order as the full walk
                const int cchunk = (nc + NBS - 1) / NBS;
                const int c0 = min(crank * cchunk, nc), c1 = min(c0 + cchunk, nc);
                if (tid == 0) s_nrel = 0;
                block_barrier();
                for (int base = c0; base < c1; base += NT) {
                    const int c = base + tid;
                    const bool rel = c < c1 && Ctr[sg.cand0 + c].x < m0;
                    const unsigned bal = __ballot_sync(0xffffffffu, rel);
                    if ((tid & 31) == 0) s_wmask[tid >> 5] = bal;
                    block_barrier();
                    int off = s_nrel + __popc(bal & ((1u << (tid & 31)) - 1u)), tot = 0;
                    for (int w = 0; w < NW; ++w) {
                        const int pc = __popc(s_wmask[w]);
                        if (w < (tid >> 5)) off += pc;
                        tot += pc;
                    }
                    if (rel && off < REL_CAP) s_rel[off] = c;
                    block_barrier();
                    if (tid == 0) s_nrel += tot;
                }
                bool over = false;  // a list that did not fit: the full walk below, every block
                double m = m0;
                if constexpr (GR) {  // the lists through global memory
                    block_barrier();
                    if (tid == 0) gxv.nrel[crank] = s_nrel;
                    for (int i = tid; i < s_nrel && i < GX_REL; i += NT) gxv.rel[(size_t)crank * GX_REL + i] = s_rel[i];
                    grid_barrier(gxv);
                    for (int r = 0; r < NBS; ++r) over |= *reinterpret_cast<volatile int *>(gxv.nrel + r) > GX_REL;
                    if (!over && tid == 0) {
                        double t_c = m0;
                        int prevk = -1;
                        for (int r = 0; r < NBS; ++r) {
                            const int n = *reinterpret_cast<volatile int *>(gxv.nrel + r);
                            const volatile int *lst = gxv.rel + (size_t)r * GX_REL;
                            for (int i = 0; i < n; ++i) {
                                const int cc = lst[i];
                                const int k = (int)((unsigned)d.cand[sg.cand0 + cc] >> 16);
                                const double2 pr = Ctr[sg.cand0 + cc];
                                if (k != prevk) { t_c = m; prevk = k; }
                                m = dmin(m, t_c <= pr.x ? t_c : pr.y);
                            }
                        }
                    }
                    grid_barrier(gxv);  // every read done before the lists are rebuilt
                } else {
                    cg::cluster_group cl = cg::this_cluster();
                    cluster_barrier();
                    for (int r = 0; r < CS; ++r) over |= *cl.map_shared_rank(&s_nrel, r) > REL_CAP;
                    if (!over && tid == 0) {
                        double t_c = m0;
                        int prevk = -1;
                        for (int r = 0; r < CS; ++r) {
                            const int n = *cl.map_shared_rank(&s_nrel, r);
                            const int *lst = cl.map_shared_rank(s_rel, r);
                            for (int i = 0; i < n; ++i) {
                                const int cc = lst[i];
                                const int k = (int)((unsigned)d.cand[sg.cand0 + cc] >> 16);
                                const double2 pr = Ctr[sg.cand0 + cc];
                                if (k != prevk) { t_c = m; prevk = k; }
                                m = dmin(m, t_c <= pr.x ? t_c : pr.y);
                            }
                        }
                    }
                    cluster_barrier();  // every remote read done before the lists are rebuilt
                }
                if (!over) return m;
            }
            double m = m0, t_c = m0;
            int prevk = -1;
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
        auto sweep = [&]() {  // kinematic nodes advanced by the step limit, ipc_contact.py:456-463
            ipc_refresh();
            double qi = 0.0;
            for (int b = sg.bc0 + gt; b < sg.bc0 + sg.nbc; b += GS) {
                const double2 q = kin_dir(d.bc_idx[b]);
                qi = dmax(qi, sqrt(q.x * q.x + q.y * q.y));
            }
            double dummy = 0.0;
            ipc_pairs(3, dummy, 1.0);
            double v[1] = {qi};
            const int ops[1] = {1};
            scene_reduce<NT, CS, 1>(v, ops, red, cres, gxp);
            const double a_tc = tc_scan(1.0);
            if (tid == 0) {
                double a_s = a_tc;
                if (v[0] > 0.0) a_s = dmin(a_s, 0.45 * d.reach / v[0]);
                S.alpha_s = a_s;
                S.q_inf = v[0];
                S.motion += dmin(a_s, 1.0) * v[0];
            }
            gsync();
            const double alpha_s = S.alpha_s;
            for (int b = sg.bc0 + gt; b < sg.bc0 + sg.nbc; b += GS) {
                const int n = d.bc_idx[b];
                const double2 tg = Tgt[b], x = xpos(n), xn = Xn[n];
                const double2 nx = alpha_s >= 1.0 ? tg : make_double2(x.x + alpha_s * (tg.x - x.x), x.y + alpha_s * (tg.y - x.y));
                const double2 xb = XBd[n];
                XD[n] = make_float2((float)(nx.x - xn.x), (float)(nx.y - xn.y));
                XR[n] = make_float2((float)(nx.x - xb.x), (float)(nx.y - xb.y));
            }
            gsync();
        };

        // the scene's step energy at x_b + r in FP64 (PNCG2DSolver._energy_into,
        // solver.py:453-498), for the line search; a kinematic node's x-hat is its position
        // (inertia 0), as the FP64 step sets it (apply_bc_kernel, IPCContact.advance_bc)
        auto energy_mx = [&]() -> double {
            double v[1] = {energy_partial(
                d, sg, gt, GS, xpos,
                [&](int n) -> double2 {
                    if (d.node_bc[n] >= 0) return xpos(n);
                    const double2 xn = Xn[n], vn = Vv[n];
                    return make_double2(xn.x + dt * d.drag * vn.x, xn.y + dt * d.drag * vn.y);
                },
                Bm, Ar, Mu, La, cols, colmu, [&](double &acc) { if (scene_ipc) ipc_pairs(2, acc, 0.0); })};
            const int ops[1] = {0};
            scene_reduce<NT, CS, 1>(v, ops, red, cres, gxp);
            return v[0];
        };

        if (scene_ipc && sg.nbc > 0) {
            sweep();
            if (tid == 0) S.pending = !(S.alpha_s >= 1.0);
            gsync();
        }

        // ================================================================ PNCG iterations (FP32)
        for (int it = 0; it < d.iter_max; ++it) {
            if (scene_ipc && S.pending) {
                sweep();
                if (tid == 0) {
                    if (S.q_inf > 0.0) S.active = 1;
                    if (it % 8 == 7) S.pending = !(S.alpha_s >= 1.0);
                }
                gsync();
            }
            if constexpr (GR) {  // a grid barrier gave up waiting: end the step with an error
                if (*reinterpret_cast<volatile int *>(gxv.err)) {
                    if (tid == 0) S.status = D2F_ESPIN;
                    break;
                }
            }
            if (!S.active && !S.pending) break;
            if (S.status != 0) break;
            if (it > 0 && it % REBASE == 0) build_base();

            // ---------------------------------------------- A1: triangles (gradient + diagonal)
            for (int t = t0 + gt; t < t1; t += GS) {
                const int i0 = __ldg(d.tri + 3 * t), i1 = __ldg(d.tri + 3 * t + 1), i2 = __ldg(d.tri + 3 * t + 2);
                const float4 B = Bm[t], du = DU0[t];
                const float A = Ar[t], mu = Mu[t], la = La[t];
                const float2 u0 = XR[i0], u1 = XR[i1], u2 = XR[i2];
                const float q1x = u1.x - u0.x, q1y = u1.y - u0.y;  // edges of x - x_b
                const float q2x = u2.x - u0.x, q2y = u2.y - u0.y;
                // displacement gradient Hn at the base x_b and its increment K (F = I + Hn + K)
                const float n00 = du.x * B.x + du.z * B.z, n01 = du.x * B.y + du.z * B.w;
                const float n10 = du.y * B.x + du.w * B.z, n11 = du.y * B.y + du.w * B.w;
                const float K00 = q1x * B.x + q2x * B.z, K01 = q1x * B.y + q2x * B.w;
                const float K10 = q1y * B.x + q2y * B.z, K11 = q1y * B.y + q2y * B.w;
                const float H00 = n00 + K00, H01 = n01 + K01, H10 = n10 + K10, H11 = n11 + K11;
                const float dH = H00 * H11 - H01 * H10;
                const float Jm1 = (H00 + H11) + dH;
                const float J = 1.f + Jm1;
                const float logJ = J > 1.0e-6f ? log1pf(Jm1) : logf(1.0e-6f);
                const float iJ = J != 0.f ? 1.f / J : 0.f;
                const float G00 = (1.f + H11) * iJ, G01 = -H10 * iJ, G10 = -H01 * iJ, G11 = (1.f + H00) * iJ;
                const float c1 = la * logJ - mu;
                // stress increment P(F) - P(Fn) from small quantities only:
                //   mu K + la (log J - log Jn) F^-T + (la log Jn - mu) (F^-T - Fn^-T),
                //   J - Jn = cof(Fn):K + det K,  F^-T - Fn^-T = (cof(K) Jn - cof(Fn) (J - Jn)) / (J Jn)
                const float Jnm1 = (n00 + n11) + (n00 * n11 - n01 * n10), Jn = 1.f + Jnm1;
                const float dJ = ((1.f + n11) * K00 - n10 * K01) + ((1.f + n00) * K11 - n01 * K10) +
                                 (K00 * K11 - K01 * K10);
                const float logJn = Jn > 1.0e-6f ? log1pf(Jnm1) : logf(1.0e-6f);
                const float dlogJ = (J > 1.0e-6f && Jn > 1.0e-6f) ? log1pf(dJ / Jn) : logJ - logJn;
                const float c1n = la * logJn - mu;
                const float iJJ = (J != 0.f && Jn != 0.f) ? 1.f / (J * Jn) : 0.f;
                const float dG00 = (K11 * Jn - (1.f + n11) * dJ) * iJJ, dG01 = (n10 * dJ - K10 * Jn) * iJJ;
                const float dG10 = (n01 * dJ - K01 * Jn) * iJJ, dG11 = (K00 * Jn - (1.f + n00) * dJ) * iJJ;
                const float ld = la * dlogJ;
                const float P00 = mu * K00 + ld * G00 + c1n * dG00;
                const float P01 = mu * K01 + ld * G01 + c1n * dG01;
                const float P10 = mu * K10 + ld * G10 + c1n * dG10;
                const float P11 = mu * K11 + ld * G11 + c1n * dG11;
                const float hA = fh2 * A;
                const float g1x = hA * (P00 * B.x + P01 * B.y), g1y = hA * (P10 * B.x + P11 * B.y);
                const float g2x = hA * (P00 * B.z + P01 * B.w), g2y = hA * (P10 * B.z + P11 * B.w);
                const float kk = la - c1;
                const float b0x = -(B.x + B.z), b0y = -(B.y + B.w);
                auto dg = [&](float bx, float by, float &dxo, float &dyo) {
                    const float bb = mu * (bx * bx + by * by);
                    const float gx = G00 * bx + G01 * by, gy = G10 * bx + G11 * by;
                    dxo = hA * fmaxf(bb + kk * gx * gx, 0.f);
                    dyo = hA * fmaxf(bb + kk * gy * gy, 0.f);
                };
                float d0x, d0y, d1x_, d1y_, d2x_, d2y_;
                dg(b0x, b0y, d0x, d0y);
                dg(B.x, B.y, d1x_, d1y_);
                dg(B.z, B.w, d2x_, d2y_);
                // accumulate at the nodes (vector atomics; the order of the FP32 sums is not fixed)
                atomicAdd(GD + i0, make_float4(-(g1x + g2x), -(g1y + g2y), d0x, d0y));
                atomicAdd(GD + i1, make_float4(g1x, g1y, d1x_, d1y_));
                atomicAdd(GD + i2, make_float4(g2x, g2y, d2x_, d2y_));
            }
            gsync();

            // ---------------------------------------------- A2: nodes (gather, colliders, friction, force)
            for (int i = n0 + gt; i < n1; i += GS) {
                Gp[i] = G[i];
                const float2 dx_ = XD[i];
                const float4 hvm = HVM[i];
                const int2 inf = NINFO[i];
                const float2 hv = make_float2(hvm.x, hvm.y);
                const float m = hvm.z;
                const int fm = inf.x & 3;
                float gx = (fm & 1) ? m * (dx_.x - hv.x) : 0.f;
                float gy = (fm & 2) ? m * (dx_.y - hv.y) : 0.f;
                float dxx = m, dyy = m;
                {
                    const float4 c = GD[i];  // the elastic sums of this iteration; reset for the next
                    GD[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                    gx += c.x; gy += c.y; dxx += c.z; dyy += c.w;
                }
                if (scene_rig) Del[i] = make_float2(dxx, dyy);
                if (inf.y >= 0) {
                    for (int k = 0; k < n_col; ++k) {
                        const Col c = cols[k];
                        float dd, nx, ny, tang = 0.f, H00 = 0.f, H11 = 0.f, gn = 1.f;
                        if (c.kind == 4) {  // half-space: phi0 (FP64 per step) + n.dx
                            nx = colf[k][0]; ny = colf[k][1];
                            dd = PHI0[(size_t)i * n_col + k] + (nx * dx_.x + ny * dx_.y);
                        } else {           // curved colliders in FP64
                            const double2 xi = xpos(i);
                            double ddd, nnx, nny, dc = 1.0;
                            SdfHit hh;
                            if (c.kind == 0) {
                                const double ex = xi.x - c.cx, ey = xi.y - c.cy;
                                dc = sqrt(ex * ex + ey * ey);
                                ddd = dc - c.r; nnx = ex / dc; nny = ey / dc;
                            } else {
                                hh = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, xi.x, xi.y);
                                ddd = hh.d; nnx = hh.gx; nny = hh.gy;
                                gn = (float)sqrt(nnx * nnx + nny * nny);
                            }
                            dd = (float)ddd; nx = (float)nnx; ny = (float)nny;
                            if (c.kind == 0) tang = 1.f / (float)dc;
                            else { H00 = (float)hh.H00; H11 = (float)hh.H11; }
                        }
                        if (dd <= 0.f || dd >= fdhat) continue;
                        const float bp = barrier_bp<float>(dd, fdhat), bpp = barrier_bpp<float>(dd, fdhat);
                        const float s = fh2 * fkappa * bp;
                        gx += s * nx; gy += s * ny;
                        float hx, hy;
                        if (c.kind == 0) {
                            const float tg = bp * tang;
                            hx = fkappa * (bpp * nx * nx + tg * (1.f - nx * nx));
                            hy = fkappa * (bpp * ny * ny + tg * (1.f - ny * ny));
                        } else {
                            hx = fkappa * (bpp * nx * nx + bp * H00);
                            hy = fkappa * (bpp * ny * ny + bp * H11);
                        }
                        dxx += fh2 * fmaxf(hx, 0.f);
                        dyy += fh2 * fmaxf(hy, 0.f);
                        if (d.friction && (fm & 3)) {  // lagged friction, slip velocity dx/dt
                            const float inx = nx / fmaxf(gn, 1e-30f), iny = ny / fmaxf(gn, 1e-30f);
                            const float f_n = fkappa * fabsf(bp) * gn;
                            const float vx = dx_.x * finv_dt, vy = dx_.y * finv_dt;
                            const float vn = vx * inx + vy * iny;
                            const float vtx = vx - vn * inx, vty = vy - vn * iny;
                            const float den = fmaxf(sqrtf(vtx * vtx + vty * vty), fepsv);
                            const float sf = fh2 * colmuf[k] * f_n;
                            if (fm & 1) gx += sf * (vtx / den);
                            if (fm & 2) gy += sf * (vty / den);
                            const float kt = sf * finv_dt / den;
                            if (fm & 1) dxx += kt * iny * iny;
                            if (fm & 2) dyy += kt * inx * inx;
                        }
                    }
                }
                const float4 g0 = G0[i];  // step-start gradient (FP32 pair) + this iteration's increments
                G[i] = make_float2(g0.x + (g0.z + gx), g0.y + (g0.w + gy));
                D[i] = make_float2(dxx, dyy);
            }
            gsync();

            // ---------------------------------------------- A3: contact between bodies, tendons (FP64)
            if (scene_ipc) {
                ipc_refresh();
                FF zf{0.f, 0.f};
                double z0 = 0.0;
                ipc_pairs32(0, zf, z0, 0.f);
                gsync();
            }
            if (sg.nten > 0) {
                // tension and stiffness of each tendon at x (Tendon.grad_diag, actuation.py:169-228)
                auto tendon_state = [&](int k, double L) {
                    double tau, keff;
                    if (d.t_stiff[k] > 0.0) {
                        const double ext = L - d.t_L0[k];
                        tau = ext > 0.0 ? d.t_stiff[k] * ext : 0.0;
                        keff = ext > 0.0 ? d.t_stiff[k] : 0.0;
                    } else {
                        tau = dmax(d.t_Tcmd[k], 0.0); keff = 0.0;
                    }
                    double *ts = d.t_state + 4 * k;
                    ts[0] = L; ts[2] = tau; ts[3] = keff;
                };
                if (sg.nten == 1) {
                    // one tendon (the common case): its length as a scene reduction over the
                    // segments, a thread per segment, instead of one thread walking them all
                    double L[1] = {0.0};
                    for (int j = sg.tent0 + gt; j < sg.tent0 + sg.ntent; j += GS) {
                        const int m = d.t_nxt[j];
                        if (m < 0) continue;
                        const double2 xa = xpos(d.t_node[j]), xb = xpos(d.t_node[m]);
                        const double ex = xb.x - xa.x, ey = xb.y - xa.y;
                        L[0] += sqrt(ex * ex + ey * ey);
                    }
                    const int ops1[1] = {0};
                    scene_reduce<NT, CS, 1>(L, ops1, red, cres, gxp);
                    if (gt == 0) tendon_state(sg.ten0, L[0]);
                } else {
                    for (int k = sg.ten0 + gt; k < sg.ten0 + sg.nten; k += GS) {
                        double L = 0.0;
                        for (int j = sg.tent0; j < sg.tent0 + sg.ntent; ++j) {
                            if (d.t_tid[j] != k) continue;
                            const int m = d.t_nxt[j];
                            if (m < 0) continue;
                            const double2 xa = xpos(d.t_node[j]), xb = xpos(d.t_node[m]);
                            const double ex = xb.x - xa.x, ey = xb.y - xa.y;
                            L += sqrt(ex * ex + ey * ey);
                        }
                        tendon_state(k, L);
                    }
                }
                gsync();
                for (int j = sg.tent0 + gt; j < sg.tent0 + sg.ntent; j += GS) {
                    const int n = d.t_node[j], k = d.t_tid[j];
                    const double tau = d.t_state[4 * k + 2], keff = d.t_state[4 * k + 3];
                    double gLx = 0, gLy = 0, geox = 0, geoy = 0;
                    const double2 xn_ = xpos(n);
                    if (d.t_prv[j] >= 0) {
                        const double2 xa = xpos(d.t_node[d.t_prv[j]]);
                        const double tx = xn_.x - xa.x, ty = xn_.y - xa.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                        const double sx = tx / ln, sy = ty / ln, il = 1.0 / ln;
                        gLx += sx; gLy += sy;
                        geox += (1.0 - sx * sx) * il; geoy += (1.0 - sy * sy) * il;
                    }
                    if (d.t_nxt[j] >= 0) {
                        const double2 xb = xpos(d.t_node[d.t_nxt[j]]);
                        const double tx = xb.x - xn_.x, ty = xb.y - xn_.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                        const double sx = tx / ln, sy = ty / ln, il = 1.0 / ln;
                        gLx -= sx; gLy -= sy;
                        geox += (1.0 - sx * sx) * il; geoy += (1.0 - sy * sy) * il;
                    }
                    // the force at x_b is in g0: add the increment since x_b
                    const double taun = d.t_state[4 * k + 1];
                    const double2 gn = tendon_dlen(xbpos, d.t_node, d.t_prv[j], d.t_nxt[j], n);
                    float *gp_ = reinterpret_cast<float *>(G + n);
                    float *dp_ = reinterpret_cast<float *>(D + n);
                    atomicAdd(gp_, (float)(h2 * (tau * gLx - taun * gn.x)));
                    atomicAdd(gp_ + 1, (float)(h2 * (tau * gLy - taun * gn.y)));
                    atomicAdd(dp_, (float)(h2 * (tau * geox + keff * gLx * gLx)));
                    atomicAdd(dp_ + 1, (float)(h2 * (tau * geoy + keff * gLy * gLy)));
                }
                gsync();
            }

            if (sg.nsp > 0 || sg.npe > 0) {
                // Springs.grad_diag (actuation.py:405-424): the force at x minus the one at x_b in
                // the base gradient (FP64), the diagonal at x
                for (int k = sg.sp0 + gt; k < sg.sp0 + sg.nsp; k += GS) {
                    const int a = d.sp_a[k], b = d.sp_b[k];
                    const double kk = d.sp_k[k], L0 = d.sp_L0[k];
                    const SpringAt sa = spring_at(xpos(a), b >= 0 ? xpos(b) : spring_anchor(d, k), kk, L0);
                    const SpringAt s0 = spring_at(XBd[a], b >= 0 ? XBd[b] : spring_anchor(d, k), kk, L0);
                    const float gx = (float)(h2 * (sa.ten * sa.nx - s0.ten * s0.nx));
                    const float gy = (float)(h2 * (sa.ten * sa.ny - s0.ten * s0.ny));
                    const float hx = (float)(h2 * (kk * sa.nx * sa.nx + sa.kt * (1.0 - sa.nx * sa.nx)));
                    const float hy = (float)(h2 * (kk * sa.ny * sa.ny + sa.kt * (1.0 - sa.ny * sa.ny)));
                    float *ga = reinterpret_cast<float *>(G + a), *da = reinterpret_cast<float *>(D + a);
                    atomicAdd(ga, gx); atomicAdd(ga + 1, gy); atomicAdd(da, hx); atomicAdd(da + 1, hy);
                    if (b >= 0) {
                        float *gb = reinterpret_cast<float *>(G + b), *db = reinterpret_cast<float *>(D + b);
                        atomicAdd(gb, -gx); atomicAdd(gb + 1, -gy); atomicAdd(db, hx); atomicAdd(db + 1, hy);
                    }
                }
                // Pressure.grad_diag (actuation.py:98-108): linear in x, so the increment since x_b
                // is the same term of the offsets r
                for (int e = sg.pe0 + gt; e < sg.pe0 + sg.npe; e += GS) {
                    const int a = d.pe_a[e], b = d.pe_b[e];
                    const float2 ra = XR[a], rb = XR[b];
                    const double sp = -0.5 * h2 * d.ch_p[d.pe_ch[e]];
                    const float gx = (float)(sp * ((double)rb.y - (double)ra.y));
                    const float gy = (float)(-sp * ((double)rb.x - (double)ra.x));
                    float *ga = reinterpret_cast<float *>(G + a), *gb = reinterpret_cast<float *>(G + b);
                    atomicAdd(ga, gx); atomicAdd(ga + 1, gy); atomicAdd(gb, gx); atomicAdd(gb + 1, gy);
                }
                gsync();
            }

            // ---------------------------------------------- A4: body-level modes
            // AffineBodies.gather, affine.py:156-175: on a cluster a warp per body (out of line);
            // in the batch kernel the block per body, inline (a call would make every thread
            // save its registers around it and double the kernel's stack frame)
            if constexpr (CL) {
                if (sg.naff > 0)
                    affine_gather(d.a_ptr, d.a_node, d.a_w, G, D, d.a_gq, d.a_gq_prev, d.a_H, sg.aff0 + (gt >> 5),
                                  sg.aff0 + sg.naff, GS / 32, tid & 31);
            } else {
                for (int b = sg.aff0; b < sg.aff0 + sg.naff; ++b) {
                    double v[18];
#pragma unroll
                    for (int q = 0; q < 18; ++q) v[q] = 0.0;
                    for (int k = d.a_ptr[b] + tid; k < d.a_ptr[b + 1]; k += NT) {
                        const int i = d.a_node[k];
                        const double *w = d.a_w + 3 * k;
                        const float2 g = G[i], dg = D[i];
                        const double gx = g.x, gy = g.y, dx = dg.x, dy = dg.y;
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
            }
            if (sg.naff > 0) {
                // the bodies' nodes take their direction from J p_q: their g leaves the node dots.
                // The zeros are written by the body entries' threads (any block of a cluster) and
                // read by the nodes' own threads in the next pass, hence the second barrier
                gsync();
                for (int k = sg.affn0 + gt; k < sg.affn0 + sg.naffn; k += GS) G[d.a_node[k]] = make_float2(0.f, 0.f);
                gsync();
            }
            if (tid == 0) { F.gPg = 0.f; F.g_Py = 0.f; F.y_Py = 0.f; }
            // one rigid piece (a free soft body): its gather is folded into the Dai-Kou pass below;
            // several pieces: one reduction each here
            const bool rig1 = sg.nrig == 1;
            for (int b = sg.rig0; !rig1 && b < sg.rig0 + sg.nrig; ++b) {  // RigidModes.gather, affine.py:404-453
                const int lb = b - sg.rig0;
                // centroid shift since the step began: sum m dx / M
                FF cs2[2] = {{0.f, 0.f}, {0.f, 0.f}};
                for (int k = sg.rign0 + gt; k < sg.rign0 + sg.nrign; k += GS) {
                    if (d.r_grp[k] != b) continue;
                    const int i = d.r_node[k];
                    const float m = HVM[i].z;
                    const float2 u = XD[i];
                    ff_add(cs2[0], m * u.x);
                    ff_add(cs2[1], m * u.y);
                }
                float nm[1] = {0.f};
                const int nmo[1] = {1};
                double so[2];
                float mo_[1];
                scene_reduce_mx<NT, CS, 2, 1>(cs2, nm, nmo, so, mo_, fred, dres, mres, cres, cmres, gxp);
                const float Mtot = (float)d.r_acc[3 * b + 2];
                const float csx = (float)so[0] / Mtot, csy = (float)so[1] / Mtot;
                FF v[11];
#pragma unroll
                for (int q = 0; q < 11; ++q) v[q] = FF{0.f, 0.f};
                for (int k = sg.rign0 + gt; k < sg.rign0 + sg.nrign; k += GS) {
                    if (d.r_grp[k] != b) continue;
                    const int i = d.r_node[k];
                    const float2 a0 = RARM[i], u = XD[i];
                    const float rx = a0.x + (u.x - csx), ry = a0.y + (u.y - csy);
                    const float2 g = G[i], gp = Gp[i], dg = D[i], de = Del[i];
                    const float m = HVM[i].z;
                    const float dx = fmaxf(dg.x - de.x, 0.f) + m, dy = fmaxf(dg.y - de.y, 0.f) + m;
                    ff_add(v[0], g.x); ff_add(v[1], g.y); ff_add(v[2], rx * g.y - ry * g.x);
                    ff_add(v[3], gp.x); ff_add(v[4], gp.y); ff_add(v[5], rx * gp.y - ry * gp.x);
                    ff_add(v[6], dx); ff_add(v[7], -dx * ry); ff_add(v[8], dy); ff_add(v[9], dy * rx);
                    ff_add(v[10], dx * ry * ry + dy * rx * rx);
                }
                double vs[11];
                scene_reduce_mx<NT, CS, 11, 1>(v, nm, nmo, vs, mo_, fred, dres, mres, cres, cmres, gxp);
                if (tid == 0) {
                    float v32[11];
                    for (int q = 0; q < 11; ++q) v32[q] = (float)vs[q];
                    rigid_precondition(v32, F, lb < 8 ? nullptr : d.r_zq + 3 * b, lb < 8 ? s_zf[lb] : nullptr);
                    RCS[b] = make_float2(csx, csy);
                    if (lb < 8) { s_cs[lb][0] = csx; s_cs[lb][1] = csy; }
                }
                gsync();
            }

            // ---------------------------------------------- B1: mask + Dai-Kou dot products
            // (+ the single rigid piece's B^T g, B^T g_prev, B^T D' B, affine.py:421-453)
            auto b2 = [&](const double *vs) {
                // affine_reduce_kernel, affine.py:178-205: each body's 6x6 solve by one thread
                // (FP64), its five Dai-Kou terms summed over the bodies in a fixed tree
                double ab[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // gPg, g.p, g.Py, y.p, y.Py of the bodies
                if constexpr (CL) {  // a thread per body, out of line
                    if (sg.naff > 0) {
                        affine_solve(d.a_q, d.a_Mu, d.a_La, d.a_gq, d.a_gq_prev, d.a_H, d.a_pq, d.a_zq, h2, sg.aff0 + gt,
                                     sg.aff0 + sg.naff, GS, ab);
                        const int ops5[5] = {0, 0, 0, 0, 0};
                        scene_reduce<NT, CS, 5>(ab, ops5, red, cres, gxp);
                    }
                } else if (tid == 0) {  // the batch kernel: thread 0, inline, 6x6 work in shared memory
                    for (int b = sg.aff0; b < sg.aff0 + sg.naff; ++b) {
                        const double *q = d.a_q + 6 * b;
                        const M2 A{q[1], q[2], q[4], q[5]};
                        const M2 Pm = nh_P(A, d.a_Mu[b], d.a_La[b]);
                        double g[6], y[6], z[6], zy[6];
                        const double hp[6] = {0.0, h2 * Pm.a, h2 * Pm.b, 0.0, h2 * Pm.c, h2 * Pm.d};
                        for (int r = 0; r < 6; ++r) g[r] = d.a_gq[6 * b + r] + hp[r];
                        reduced_hessian(A, d.a_Mu[b], d.a_La[b], h2, d.a_H + 18 * b, s_H6);
                        chol6(s_H6, s_L6);
                        for (int r = 0; r < 6; ++r) y[r] = g[r] - d.a_gq_prev[6 * b + r];
                        chol6_solve(s_L6, g, z);
                        chol6_solve(s_L6, y, zy);
                        const double *pq = d.a_pq + 6 * b;
                        for (int r = 0; r < 6; ++r) {
                            ab[0] += g[r] * z[r]; ab[1] += g[r] * pq[r]; ab[2] += g[r] * zy[r];
                            ab[3] += y[r] * pq[r]; ab[4] += y[r] * zy[r];
                        }
                        for (int r = 0; r < 6; ++r) { d.a_gq[6 * b + r] = g[r]; d.a_zq[6 * b + r] = z[r]; }
                    }
                }
                if (tid == 0) {  // B2: Dai-Kou beta (every block of a cluster alike)
                    // the dot products and the coefficients formed from them in FP64 (the
                    // rigid pieces' terms come from the FP32 preconditioner solve); divisions by
                    // rcp64, in an order with no product of two dot products
                    double gPg = vs[0] + (double)F.gPg, g_p = vs[1], g_Py = vs[2] + (double)F.g_Py;
                    double y_p = vs[3], y_Py = vs[4] + (double)F.y_Py;
                    if (sg.naff > 0) { gPg += ab[0]; g_p += ab[1]; g_Py += ab[2]; y_p += ab[3]; y_Py += ab[4]; }
                    double bta = 0.0;  // finalize_beta_kernel, kernels.py:195-217
                    if (it > 0 && dabs(y_p) > 1.0e-30) {
                        const double r = rcp64(y_p);
                        bta = (g_Py - y_Py * (g_p * r)) * r;
                    }
                    double gtp = -gPg + bta * g_p;
                    if (gtp >= 0.0) { bta = 0.0; gtp = -gPg; }
                    if (use_guard && it > 0) {  // cg_guard_kernel, solver.py:76-94
                        const bool hold = scene_ipc && S.pending && S.q_inf > 0.0;
                        if (!hold && y_p < d.cg_guard * S.alpha * S.pHp) { bta = 0.0; gtp = -gPg; }
                    }
                    S.beta = bta; S.gTp = gtp; F.beta = (float)bta; F.gn2 = (float)vs[5];
                }
                gsync();
                if (sg.naff > 0) {  // the bodies' directions, read by B3 (FP64 beta: the stiff bodies need it)
                    const double bta = S.beta;
                    for (int b = sg.aff0 + gt; b < sg.aff0 + sg.naff; b += GS)
                        for (int r = 0; r < 6; ++r) d.a_pq[6 * b + r] = -d.a_zq[6 * b + r] + bta * d.a_pq[6 * b + r];
                    gsync();
                }
            };
            auto b1 = [&](auto rig_tag) {
                // the five Dai-Kou dots and |g|^2 as compensated sums; the rigid piece's
                // projections (they shape the preconditioner only) as plain FP32 sums
                constexpr bool RIG = decltype(rig_tag)::value;
                constexpr int NS = 6, NM = RIG ? 12 : 1;
                FF v[NS];
#pragma unroll
                for (int q = 0; q < NS; ++q) v[q] = FF{0.f, 0.f};
                float r[NM];
                int rops[NM];
#pragma unroll
                for (int q = 0; q < NM; ++q) { r[q] = 0.f; rops[q] = q == 0 ? 1 : 0; }
                const float csx = F.csx, csy = F.csy;
                for (int i = n0 + gt; i < n1; i += GS) {
                    const int inf = NINFO[i].x, fm = inf & 3;
                    float2 g = G[i];
                    const float2 dg = D[i], gp = Gp[i], pp = P[i];
                    if constexpr (RIG) {
                        if (inf & NI_RIG) {  // a free node: the mask does not change g
                            const float2 a0 = RARM[i], u = XD[i], de = Del[i];
                            const float rx = a0.x + (u.x - csx), ry = a0.y + (u.y - csy);
                            const float m = HVM[i].z;
                            const float dx = fmaxf(dg.x - de.x, 0.f) + m, dy = fmaxf(dg.y - de.y, 0.f) + m;
                            r[1] += g.x; r[2] += g.y; r[3] += rx * g.y - ry * g.x;
                            r[4] += gp.x; r[5] += gp.y; r[6] += rx * gp.y - ry * gp.x;
                            r[7] += dx; r[8] += -dx * ry; r[9] += dy; r[10] += dy * rx;
                            r[11] += dx * ry * ry + dy * rx * rx;
                        }
                    }
                    if (!(fm & 1)) g.x = 0.f;
                    if (!(fm & 2)) g.y = 0.f;
                    G[i] = g;
                    const float Px = (fm & 1) ? 1.f / fmaxf(dg.x, 1.0e-12f) : 0.f;
                    const float Py = (fm & 2) ? 1.f / fmaxf(dg.y, 1.0e-12f) : 0.f;
                    const float yx = g.x - gp.x, yy = g.y - gp.y;
                    const float Pg0 = Px * g.x, Pg1 = Py * g.y, Py0 = Px * yx, Py1 = Py * yy;
                    ff_add(v[0], g.x * Pg0 + g.y * Pg1);
                    ff_add(v[1], g.x * pp.x + g.y * pp.y);
                    ff_add(v[2], g.x * Py0 + g.y * Py1);
                    ff_add(v[3], yx * pp.x + yy * pp.y);
                    ff_add(v[4], yx * Py0 + yy * Py1);
                    ff_add(v[5], g.x * g.x + g.y * g.y);
                }
                double vs[NS];
                float mo_[NM];
                scene_reduce_mx<NT, CS, NS, NM>(v, r, rops, vs, mo_, fred, dres, mres, cres, cmres, gxp);
                if constexpr (RIG) {
                    if (tid == 0) {  // rigid_reduce_kernel, affine.py:456-473
                        rigid_precondition(mo_ + 1, F, nullptr, s_zf[0]);
                        s_cs[0][0] = csx; s_cs[0][1] = csy;
                    }
                }
                b2(vs);
            };
            if (rig1) b1(std::true_type{}); else b1(std::false_type{});

            // ---------------------------------------------- B3: direction + node curvature and caps
            FF acc_pHp{0.f, 0.f}, acc_mpx{0.f, 0.f}, acc_mpy{0.f, 0.f};  // p^T H p; single rigid piece: sum m p
            double acc_rare = 0.0;
            float acc_pinf = 0.f, acc_clr = 1.0e30f, acc_alpha = falpha_max;
            {
                const float bta = F.beta;
                for (int i = n0 + gt; i < n1; i += GS) {
                    const int2 inf = NINFO[i];
                    const int fm = inf.x & 3;
                    const float2 dx_ = XD[i];
                    const float mi = HVM[i].z;
                    float px, py;
                    if (inf.x & NI_AFF) {
                        const int ka = d.node_aff[i];
                        const double *w = d.a_w + 3 * ka, *pq = d.a_pq + 6 * d.a_grp[ka];
                        px = (float)(w[0] * pq[0] + w[1] * pq[1] + w[2] * pq[2]);
                        py = (float)(w[0] * pq[3] + w[1] * pq[4] + w[2] * pq[5]);
                    } else {
                        const float2 g = G[i], dg = D[i], po = P[i];
                        px = (fm & 1) ? -g.x / fmaxf(dg.x, 1.0e-12f) + bta * po.x : 0.f;
                        py = (fm & 2) ? -g.y / fmaxf(dg.y, 1.0e-12f) + bta * po.y : 0.f;
                        if (inf.x & NI_RIG) {
                            int lb = (inf.x >> 4) & 15;
                            if (lb == 15) lb = d.r_grp[d.node_rig[i]] - sg.rig0;
                            float z0, z1, z2, csx, csy;
                            if (lb < 8) {
                                z0 = s_zf[lb][0]; z1 = s_zf[lb][1]; z2 = s_zf[lb][2]; csx = s_cs[lb][0]; csy = s_cs[lb][1];
                            } else {
                                const double *z = d.r_zq + 3 * (sg.rig0 + lb);
                                const float2 cs = RCS[sg.rig0 + lb];
                                z0 = (float)z[0]; z1 = (float)z[1]; z2 = (float)z[2]; csx = cs.x; csy = cs.y;
                            }
                            const float2 a0 = RARM[i];
                            const float rx = a0.x + (dx_.x - csx), ry = a0.y + (dx_.y - csy);
                            px -= z0 - z2 * ry;
                            py -= z1 + z2 * rx;
                        }
                    }
                    P[i] = make_float2(px, py);
                    ff_add(acc_pHp, mi * (px * px + py * py));
                    if (rig1 && (inf.x & NI_RIG)) { ff_add(acc_mpx, mi * px); ff_add(acc_mpy, mi * py); }
                    acc_pinf = fmaxf(acc_pinf, sqrtf(px * px + py * py));
                    if (inf.y >= 0) {
                        for (int k = 0; k < n_col; ++k) {
                            const Col c = cols[k];
                            if (c.kind == 4) {  // half-space: clearance, CCD, barrier and friction curvature
                                const float nx = colf[k][0], ny = colf[k][1];
                                const float dd = PHI0[(size_t)i * n_col + k] + (nx * dx_.x + ny * dx_.y);
                                const float gp = nx * px + ny * py;
                                if (!(gp >= 0.f || dd <= 0.f)) acc_alpha = fminf(acc_alpha, feta * dd / (-gp));
                                acc_clr = fminf(acc_clr, dd);
                                if (dd <= 0.f || dd >= fdhat) continue;
                                const float bp = barrier_bp<float>(dd, fdhat), bpp = barrier_bpp<float>(dd, fdhat);
                                ff_add(acc_pHp, fh2 * fmaxf(fkappa * (bpp * gp * gp), 0.f));
                                if (d.friction && (fm & 3)) {
                                    const float f_n = fkappa * fabsf(bp);
                                    const float vx = dx_.x * finv_dt, vy = dx_.y * finv_dt;
                                    const float vn = vx * nx + vy * ny;
                                    const float vtx = vx - vn * nx, vty = vy - vn * ny;
                                    const float den = fmaxf(sqrtf(vtx * vtx + vty * vty), fepsv);
                                    const float kt = fh2 * colmuf[k] * f_n * finv_dt / den;
                                    const float pt = ((fm & 1) ? px : 0.f) * (-ny) + ((fm & 2) ? py : 0.f) * nx;
                                    ff_add(acc_pHp, kt * pt * pt);
                                }
                                continue;
                            }
                            // curved colliders, FP64
                            const double2 xi = xpos(i);
                            double dd, nx, ny, dc = 1.0, gn = 1.0;
                            SdfHit hh;
                            if (c.kind == 0) {
                                const double ex = xi.x - c.cx, ey = xi.y - c.cy;
                                dc = sqrt(ex * ex + ey * ey);
                                dd = dc - c.r; nx = ex / dc; ny = ey / dc;
                                const double a = (double)px * px + (double)py * py;
                                if (a >= 1.0e-24) {  // disc_ccd_kernel, kernels.py:344-371
                                    const double bq = 2.0 * (ex * px + ey * py), cq = (ex * ex + ey * ey) - c.r * c.r;
                                    const double disc = bq * bq - 4.0 * a * cq;
                                    if (disc >= 0.0) {
                                        const double sq = sqrt(disc), r1 = (-bq - sq) / (2.0 * a), r2 = (-bq + sq) / (2.0 * a);
                                        double sv = BIG;
                                        if (r1 > 0.0) sv = dmin(sv, r1);
                                        if (r2 > 0.0) sv = dmin(sv, r2);
                                        if (sv < BIG) acc_alpha = fminf(acc_alpha, (float)(d.ccd_eta * sv));
                                    }
                                }
                            } else {
                                hh = sdf_eval(c.kind, c.cx, c.cy, c.rx, c.ry, c.rref, xi.x, xi.y);
                                dd = hh.d; nx = hh.gx; ny = hh.gy;
                                gn = sqrt(nx * nx + ny * ny);
                                const double gp = nx * px + ny * py;
                                if (!(gp >= 0.0 || dd <= 0.0)) acc_alpha = fminf(acc_alpha, (float)(d.ccd_eta * dd / (-gp)));
                            }
                            acc_clr = fminf(acc_clr, (float)dd);
                            if (dd <= 0.0 || dd >= dhat) continue;
                            const float rd = (float)dd, rnx = (float)nx, rny = (float)ny;
                            const float bp = barrier_bp<float>(rd, fdhat), bpp = barrier_bpp<float>(rd, fdhat);
                            float val;
                            if (c.kind == 0) {
                                const float pn = px * rnx + py * rny;
                                const float ptx = px - pn * rnx, pty = py - pn * rny;
                                val = fkappa * (bpp * pn * pn + (bp / (float)dc) * (ptx * ptx + pty * pty));
                            } else {
                                const float gp = rnx * px + rny * py;
                                const float Hp0 = (float)hh.H00 * px + (float)hh.H01 * py, Hp1 = (float)hh.H10 * px + (float)hh.H11 * py;
                                val = fkappa * (bpp * gp * gp + bp * (px * Hp0 + py * Hp1));
                            }
                            ff_add(acc_pHp, fh2 * fmaxf(val, 0.f));
                            if (d.friction && (fm & 3)) {
                                const float ig = 1.f / fmaxf((float)gn, 1e-30f);
                                const float nnx = rnx * ig, nny = rny * ig;
                                const float f_n = fkappa * fabsf(bp) * (float)gn;
                                const float vx = dx_.x * finv_dt, vy = dx_.y * finv_dt;
                                const float vn = vx * nnx + vy * nny;
                                const float vtx = vx - vn * nnx, vty = vy - vn * nny;
                                const float den = fmaxf(sqrtf(vtx * vtx + vty * vty), fepsv);
                                const float kt = fh2 * colmuf[k] * f_n * finv_dt / den;
                                const float pt = ((fm & 1) ? px : 0.f) * (-nny) + ((fm & 2) ? py : 0.f) * nnx;
                                ff_add(acc_pHp, kt * pt * pt);
                            }
                        }
                    }
                }
            }
            gsync();

            // ---------------------------------------------- B4: triangles (curvature + inversion cap)
            {
                const float shrink = (float)d.area_shrink;
                for (int t = t0 + gt; t < t1; t += GS) {
                    const int i0 = __ldg(d.tri + 3 * t), i1 = __ldg(d.tri + 3 * t + 1), i2 = __ldg(d.tri + 3 * t + 2);
                    const float2 p0 = P[i0], p1 = P[i1], p2 = P[i2];
                    const float2 u0 = XR[i0], u1 = XR[i1], u2 = XR[i2];
                    const float4 B = Bm[t], du = DU0[t];
                    const float A = Ar[t], mu = Mu[t], la = La[t];
                    // F^-T and la log J - mu at x, formed again here rather than cached by the
                    // gradient pass (36 bytes a triangle less to write and read each iteration)
                    const float d1x = du.x + (u1.x - u0.x), d1y = du.y + (u1.y - u0.y);
                    const float d2x = du.z + (u2.x - u0.x), d2y = du.w + (u2.y - u0.y);
                    const float H00 = d1x * B.x + d2x * B.z, H01 = d1x * B.y + d2x * B.w;
                    const float H10 = d1y * B.x + d2y * B.z, H11 = d1y * B.y + d2y * B.w;
                    const float dH = H00 * H11 - H01 * H10, Jm1 = (H00 + H11) + dH, J = 1.f + Jm1;
                    const float logJ = J > 1.0e-6f ? log1pf(Jm1) : logf(1.0e-6f);
                    const float iJ = J != 0.f ? 1.f / J : 0.f;
                    const float G00 = (1.f + H11) * iJ, G01 = -H10 * iJ, G10 = -H01 * iJ, G11 = (1.f + H00) * iJ;
                    const float c1 = la * logJ - mu;
                    // current edge vectors: rest edges (the columns of B^-1) + displacement edges
                    const float idet = 1.f / (B.x * B.w - B.y * B.z);
                    const float e1x = B.w * idet + d1x, e1y = -B.z * idet + d1y;
                    const float e2x = -B.y * idet + d2x, e2y = B.x * idet + d2y;
                    const float q1x = p1.x - p0.x, q1y = p1.y - p0.y, q2x = p2.x - p0.x, q2y = p2.y - p0.y;
                    const float f00 = q1x * B.x + q2x * B.z, f01 = q1x * B.y + q2x * B.w;
                    const float f10 = q1y * B.x + q2y * B.z, f11 = q1y * B.y + q2y * B.w;
                    const float dd = f00 * f00 + f01 * f01 + f10 * f10 + f11 * f11;
                    const float GdF = G00 * f00 + G01 * f01 + G10 * f10 + G11 * f11;
                    const float M00 = f00 * G00 + f10 * G10, M01 = f00 * G01 + f10 * G11;
                    const float M10 = f01 * G00 + f11 * G10, M11 = f01 * G01 + f11 * G11;
                    const float tr = M00 * M00 + 2.f * M01 * M10 + M11 * M11;
                    ff_add(acc_pHp, fh2 * fmaxf(A * (mu * dd + la * GdF * GdF - c1 * tr), 0.f));
                    const float a0 = e1x * e2y - e1y * e2x;  // inversion_alpha_kernel, kernels.py:303-341
                    const float a1 = (e1x * q2y - e1y * q2x) + (q1x * e2y - q1y * e2x);
                    const float a2 = q1x * q2y - q1y * q2x;
                    const float cc = a0 - shrink * a0;
                    if (fabsf(a2) < 1.0e-24f) {
                        if (fabsf(a1) > 1.0e-24f) {
                            const float s = -cc / a1;
                            if (s > 0.f) acc_alpha = fminf(acc_alpha, s);
                        }
                    } else {
                        const float disc = a1 * a1 - 4.f * a2 * cc;
                        if (disc >= 0.f) {
                            const float sq = sqrtf(disc);
                            const float r1 = (-a1 - sq) / (2.f * a2), r2 = (-a1 + sq) / (2.f * a2);
                            if (r1 > 0.f) acc_alpha = fminf(acc_alpha, r1);
                            if (r2 > 0.f) acc_alpha = fminf(acc_alpha, r2);
                        }
                    }
                }
                if (scene_rare) {
                    for (int b = sg.aff0 + gt; b < sg.aff0 + sg.naff; b += GS) {  // affine_pHp_kernel
                        const double *q = d.a_q + 6 * b, *pq = d.a_pq + 6 * b;
                        const M2 dA{pq[1], pq[2], pq[4], pq[5]}, A{q[1], q[2], q[4], q[5]};
                        acc_rare += h2 * dmax(ddot2(dA, nh_d2(A, dA, d.a_Mu[b], d.a_La[b])), 0.0);
                    }
                    if (scene_ipc) ipc_pairs32(1, acc_pHp, acc_rare, falpha_max);
                    for (int k = sg.sp0 + gt; k < sg.sp0 + sg.nsp; k += GS) {  // Springs.pHp, actuation.py:427-444
                        const int a = d.sp_a[k], b = d.sp_b[k];
                        const SpringAt sa = spring_at(xpos(a), b >= 0 ? xpos(b) : spring_anchor(d, k), d.sp_k[k], d.sp_L0[k]);
                        double dpx = (double)P[a].x, dpy = (double)P[a].y;
                        if (b >= 0) { dpx -= (double)P[b].x; dpy -= (double)P[b].y; }
                        const double along = dpx * sa.nx + dpy * sa.ny;
                        acc_rare += h2 * (d.sp_k[k] * along * along + sa.kt * ((dpx * dpx + dpy * dpy) - along * along));
                    }
                    for (int e = sg.pe0 + gt; e < sg.pe0 + sg.npe; e += GS) {  // Pressure.pHp, actuation.py:111-118
                        const float2 pa = P[d.pe_a[e]], pb = P[d.pe_b[e]];
                        acc_rare += -h2 * d.ch_p[d.pe_ch[e]] * ((double)pa.x * (double)pb.y - (double)pa.y * (double)pb.x);
                    }
                    const bool ten_par = sg.nten == 1 && d.t_state[4 * sg.ten0 + 3] == 0.0;
                    if (ten_par) {
                        // one tendon without length stiffness at x (Tendon.pHp): a thread per
                        // segment, tau / len (|dp|^2 - (dp.s)^2) each
                        const double tau = d.t_state[4 * sg.ten0 + 2];
                        for (int j = sg.tent0 + gt; j < sg.tent0 + sg.ntent; j += GS) {
                            const int m = d.t_nxt[j];
                            if (m < 0) continue;
                            const int na = d.t_node[j], nb_ = d.t_node[m];
                            const double2 xa = xpos(na), xb = xpos(nb_);
                            const double tx = xb.x - xa.x, ty = xb.y - xa.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                            const double sx = tx / ln, sy = ty / ln;
                            const float2 pa = P[na], pb = P[nb_];
                            const double dpx = (double)pb.x - (double)pa.x, dpy = (double)pb.y - (double)pa.y;
                            const double along = dpx * sx + dpy * sy;
                            acc_rare += h2 * tau * ((dpx * dpx + dpy * dpy) - along * along) * (1.0 / ln);
                        }
                    }
                    for (int k = sg.ten0 + gt; !ten_par && k < sg.ten0 + sg.nten; k += GS) {  // Tendon.pHp, a thread per tendon
                        const double tau = d.t_state[4 * k + 2], keff = d.t_state[4 * k + 3];
                        double dL = 0.0;
                        for (int j = sg.tent0; j < sg.tent0 + sg.ntent; ++j) {
                            if (d.t_tid[j] != k) continue;
                            const int m = d.t_nxt[j];
                            if (m < 0) continue;
                            const int na = d.t_node[j], nb_ = d.t_node[m];
                            const double2 xa = xpos(na), xb = xpos(nb_);
                            const double tx = xb.x - xa.x, ty = xb.y - xa.y, ln = dmax(sqrt(tx * tx + ty * ty), 1.0e-12);
                            const double sx = tx / ln, sy = ty / ln;
                            const float2 pa = P[na], pb = P[nb_];
                            const double dpx = (double)pb.x - (double)pa.x, dpy = (double)pb.y - (double)pa.y;
                            const double along = dpx * sx + dpy * sy;
                            dL += along;
                            acc_rare += h2 * tau * ((dpx * dpx + dpy * dpy) - along * along) * (1.0 / ln);
                        }
                        acc_rare += h2 * keff * dL * dL;
                    }
                    // FP64 contributions of the rare terms joined into the compensated pair
                    const float hi = (float)acc_rare;
                    ff_add(acc_pHp, hi);
                    ff_add(acc_pHp, (float)(acc_rare - (double)hi));
                }
            }
            {
                FF sv[3] = {acc_pHp, acc_mpx, acc_mpy};
                float mv[3] = {acc_pinf, acc_clr, acc_alpha};
                const int mops[3] = {1, 2, 2};
                double so[3];
                float mo[3];
                scene_reduce_mx<NT, CS, 3, 3>(sv, mv, mops, so, mo, fred, dres, mres, cres, cmres, gxp);
                const double a_ccd = scene_ipc ? tc_scan(d.alpha_max) : 0.0;
                // ---------------------------------------------- B5: step length and convergence
                // (alpha_finalize_kernel, kernels.py:374-423): the step length and the
                // energy-decrease test in FP64 from the FP64 dot products, the caps and the
                // gradient-norm test in FP32
                if (tid == 0) {
                    const double ph = so[0];
                    const float pinf = mo[0], clr = mo[1];
                    float af = mo[2];
                    if (scene_ipc) {
                        af = fminf(af, __double2float_rd(a_ccd));
                        if (pinf > 0.f) af = fminf(af, freach45 / pinf);
                    }
                    F.pinf = pinf;
                    S.pHp = ph;
                    double a = af;
                    S.alpha = a;
                    if (S.active) {
                        bool done = false;
                        if (use_gtol) {
                            if (it == 0) F.gn0 = F.gn2;
                            else if (F.gn2 <= fgtol2 * F.gn0) { S.active = 0; done = true; }
                        }
                        if (!done) {
                            if (ph > 0.0) a = dmin(a, -S.gTp * rcp64(ph));
                            if (clr < fnear && pinf > 0.f) a = dmin(a, (double)(0.5f * fdhat / pinf));
                            if (!(a == a)) { S.status = D2F_ENAN; S.active = 0; S.alpha = 0.0; }
                            else if (a <= 0.0) { S.active = 0; S.alpha = 0.0; }
                            else {
                                S.alpha = a;
                                if (use_tolx && (float)a * pinf < ftol_x) { S.active = 0; S.iters += 1; }
                                else {
                                    const double dm = a * (-S.gTp - 0.5 * a * ph);
                                    if (it == 0) S.dE0 = dmax(dm, 1.0e-300);
                                    else if (dm < d.eps * S.dE0) S.active = 0;
                                    S.iters += 1;
                                }
                            }
                        }
                    }
                    F.alpha = (float)S.alpha;
                    if (S.active) {
                        if (scene_ipc) S.motion += S.alpha * (double)pinf;  // bound on any node's move
                        if (rig1) {                              // centroid shift, sum m dx / M
                            const float mx = (float)so[1] * F.inv_m, my = (float)so[2] * F.inv_m;
                            if (line_search) {                   // added with the accepted step
                                F.mpx = mx;
                                F.mpy = my;
                            } else {
                                S.csx += S.alpha * (double)mx;
                                S.csy += S.alpha * (double)my;
                                F.csx = (float)S.csx;
                                F.csy = (float)S.csy;
                            }
                        }
                    }
                }
                gsync();
                if (sg.naff > 0 && S.active && !line_search) {  // AffineBodies.advance, affine.py:249-257: q += alpha p_q
                    for (int b = sg.aff0 + gt; b < sg.aff0 + sg.naff; b += GS)
                        for (int r = 0; r < 6; ++r) d.a_q[6 * b + r] += S.alpha * d.a_pq[6 * b + r];
                    gsync();
                }
            }

            // ---------------------------------------------- D1: r += alpha p, dx = (x_b - x_n) + r (slaved nodes: J q),
            // or the backtracking line search (solver.py:397-425): the energy E0 at x in FP64,
            // then n_backtrack trial points x_b + (r0 + alpha p) (affine bodies q0 + alpha p_q,
            // affine.py:383-389), alpha halved while E exceeds E0 + ls_tol (|E0| + 1)
            // (ls_halve_kernel, solver.py:63-73). The trial points lie within alpha |p|_inf of x,
            // which S.motion already counts, so one candidate-list check before the first trial
            // covers them all (a rebuild there is at x; the far cap keeps alpha |p|_inf within
            // 0.45 reach < skin / 2 of it).
            if (line_search) {
                float2 *__restrict__ R0 = reinterpret_cast<float2 *>(d.xu);
                double *__restrict__ Q0 = d.xu + 2 * (size_t)d.N;
                const double E0 = energy_mx();
                for (int i = n0 + gt; i < n1; i += GS) R0[i] = XR[i];
                for (int k = sg.aff0 * 6 + gt; k < (sg.aff0 + sg.naff) * 6; k += GS) Q0[k] = d.a_q[k];
                if (scene_ipc) {
                    const bool rebuild = S.rebuild || 2.0 * S.motion >= d.skin;
                    ipc_refresh();
                    if (rebuild) {  // rebuilt at x: the trial points are within alpha |p|_inf of it
                        if (tid == 0) S.motion = S.alpha * (double)F.pinf;
                        gsync();
                    }
                    ipc_far = S.dmin_c - 2.0 * S.motion >= d.reach;
                }
                gsync();
                auto trial = [&]() {  // set_x_from_x0_kernel (solver.py:52-60) + affine_trial_kernel
                    if (S.active) {
                        const double al = S.alpha;
                        const float alf = F.alpha;
                        for (int k = sg.aff0 * 6 + gt; k < (sg.aff0 + sg.naff) * 6; k += GS)
                            d.a_q[k] = Q0[k] + al * d.a_pq[k];
                        if (sg.naff > 0) gsync();
                        for (int i = n0 + gt; i < n1; i += GS) {
                            if (NINFO[i].x & NI_AFF) {
                                const int ka = d.node_aff[i];
                                const double *w = d.a_w + 3 * ka, *q = d.a_q + 6 * d.a_grp[ka];
                                const double2 xn = Xn[i], xb = XBd[i];
                                const double jx = w[0] * q[0] + w[1] * q[1] + w[2] * q[2];
                                const double jy = w[0] * q[3] + w[1] * q[4] + w[2] * q[5];
                                XD[i] = make_float2((float)(jx - xn.x), (float)(jy - xn.y));
                                XR[i] = make_float2((float)(jx - xb.x), (float)(jy - xb.y));
                            } else {
                                const float2 pp = P[i], r = R0[i], db = DB[i];
                                const float2 rn = make_float2(r.x + alf * pp.x, r.y + alf * pp.y);
                                XR[i] = rn;
                                XD[i] = make_float2(db.x + rn.x, db.y + rn.y);
                            }
                        }
                    }
                    gsync();
                };
                for (int bt = 0; bt < d.n_backtrack; ++bt) {
                    trial();
                    const double E = energy_mx();
                    if (tid == 0 && S.active && E > E0 + d.ls_tol * (dabs(E0) + 1.0)) { S.alpha *= 0.5; F.alpha *= 0.5f; }
                    gsync();
                }
                trial();
                if (tid == 0 && S.active && sg.nrig == 1) {
                    S.csx += S.alpha * (double)F.mpx;
                    S.csy += S.alpha * (double)F.mpy;
                    F.csx = (float)S.csx;
                    F.csy = (float)S.csy;
                }
                gsync();
            } else {
                const bool act = S.active != 0;
                const float al = F.alpha;
                for (int i = n0 + gt; i < n1; i += GS) {
                    if (NINFO[i].x & NI_AFF) {
                        const int ka = d.node_aff[i];
                        const double *w = d.a_w + 3 * ka, *q = d.a_q + 6 * d.a_grp[ka];
                        const double2 xn = Xn[i], xb = XBd[i];
                        const double jx = w[0] * q[0] + w[1] * q[1] + w[2] * q[2];
                        const double jy = w[0] * q[3] + w[1] * q[4] + w[2] * q[5];
                        XD[i] = make_float2((float)(jx - xn.x), (float)(jy - xn.y));
                        XR[i] = make_float2((float)(jx - xb.x), (float)(jy - xb.y));
                    } else if (act) {
                        const float2 pp = P[i], r = XR[i], db = DB[i];
                        const float2 rn = make_float2(r.x + al * pp.x, r.y + al * pp.y);
                        XR[i] = rn;
                        XD[i] = make_float2(db.x + rn.x, db.y + rn.y);
                    }
                }
                gsync();
            }
        }

        // ================================================================ commit (FP64)
        for (int i = n0 + gt; i < n1; i += GS) {
            const double2 xn = Xn[i];
            const double2 xi = xpos(i);
            X[i] = xi;
            Vv[i] = make_double2((xi.x - xn.x) * inv_dt, (xi.y - xn.y) * inv_dt);
        }
        if (tid == 0 && crank == 0) {
            d.iters[sc] = S.iters;
            d.active[sc] = S.active;
            d.status[sc] = S.status;
        }
        gsync();
    }
}

}  // namespace d2f
