// d2f_capi.cu — the C ABI of include/d2f.h: descriptor validation, launch shape, the
// entry points, and the no-allocation step with its static scratch.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pncg_kernel.cuh"
#include <stdio.h>
#include <string.h>

#include "d2f_solver.h"

thread_local char g_err[512];

int d2f_fail(int code, const char *msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return code;
}
static int fail(int code, const char *msg) { return d2f_fail(code, msg); }

// The built variant for (threads, blocks_per_sm): an exact match, else the first variant of
// that width, else (128, 4).
static void pick_variant(int nt, int bps, int *vnt, int *vminb) {
    int fnt = 0, fmb = 0;
#define D2F_PICK(N, MB)                               \
    if (N == nt && MB == bps) { *vnt = N; *vminb = MB; return; } \
    if (N == nt && !fnt) { fnt = N; fmb = MB; }
    D2F_VARIANTS(D2F_PICK)
#undef D2F_PICK
    if (fnt) { *vnt = fnt; *vminb = fmb; return; }
    *vnt = 128;
    *vminb = 4;
}

// Threads per scene block when the caller leaves it to the library: 256 when the batch has
// at most two scenes per SM (few blocks: each needs more threads to hide latency), else 128.
int d2f_default_threads(const d2f_scene_desc &d) {
    if (d.threads) return d.threads;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 128;
    return d.n_scenes <= 2 * nsm ? 256 : 128;
}

static int occupancy(const d2f_scene_desc &d, int smem, int vnt, int vminb) {
    return d.precision == D2F_MIXED ? d2f::occupancy_mixed(vnt, vminb, smem, d2f::mixed_features(d)) : d2f::occupancy_fp64(vnt, vminb, smem);
}

extern "C" {

int32_t d2f_abi_version(void) { return D2F_ABI_VERSION; }

const char *d2f_last_error(void) { return g_err; }

}  // extern "C"

// Checks every size and pointer of a descriptor; the scratch pointers (escr, ecache, cand,
// xref, work) only when `scratch` is set.
static int validate(const d2f_scene_desc &d, bool scratch) {
    if (d.abi_version != D2F_ABI_VERSION) return fail(D2F_EINVAL, "d2f: ABI version mismatch");
    if (d.precision != D2F_FP64 && d.precision != D2F_MIXED) return fail(D2F_EINVAL, "d2f: unknown precision mode");
    if (d.n_scenes <= 0 || d.N <= 0 || d.T <= 0) return fail(D2F_EINVAL, "d2f: empty scene");
    if (d.n_col < 0 || d.n_col > d2f::MAX_COL) return fail(D2F_EINVAL, "d2f: at most 16 colliders");
    if (!d.segs || !d.x || !d.v || !d.xn || !d.xhat || !d.grad || !d.grad_prev || !d.p || !d.diagH ||
        !d.mass || !d.free_mask || !d.inc_ptr || !d.inc || !d.node_bslot || !d.node_bc || !d.node_aff ||
        !d.node_rig || !d.tri || !d.Bm || !d.area || !d.mu || !d.lam || !d.iters || !d.active || !d.status)
        return fail(D2F_EINVAL, "d2f: a required device pointer is null");
    if (scratch && (!d.escr || !d.ecache || !d.work)) return fail(D2F_EINVAL, "d2f: a scratch pointer is null");
    if (d.precision == D2F_MIXED && (!d.xrest || !d.Dm))
        return fail(D2F_EINVAL, "d2f: mixed precision needs xrest and Dm");
    if (d.precision == D2F_MIXED && scratch && !d.mscr) return fail(D2F_EINVAL, "d2f: mixed precision needs mscr");
    if (d.Nb > 0 && !d.bnd) return fail(D2F_EINVAL, "d2f: boundary nodes without bnd[]");
    if (d.n_col > 0 && !d.colliders) return fail(D2F_EINVAL, "d2f: colliders pointer is null");
    if (d.n_bc > 0 && (!d.bc_idx || !d.bc_target)) return fail(D2F_EINVAL, "d2f: kinematic arrays missing");
    if (d.Ne > 0 && (!d.ea || !d.eb || !d.ela || !d.elb || !d.ca || !d.cb || !d.excl_ptr || !d.excl_idx ||
                     d.cand_total <= 0))
        return fail(D2F_EINVAL, "d2f: IPC arrays missing");
    if (d.Ne > 0 && scratch && (!d.cand || !d.cand_tr || !d.xref)) return fail(D2F_EINVAL, "d2f: IPC scratch missing");
    if (d.Ne > 0 && (d.max_nb <= 0 || d.max_nb > 24 * 1024))
        return fail(D2F_EINVAL, "d2f: max_nb must be in 1..24576 with IPC contact");
    if (d.n_rig > 0 && (!d.diag_el || !d.r_node || !d.r_grp || !d.r_acc || !d.r_zq))
        return fail(D2F_EINVAL, "d2f: rigid-mode arrays missing");
    if (d.n_aff > 0 && (!d.a_node || !d.a_grp || !d.a_ptr || !d.a_w || !d.a_Mu || !d.a_La || !d.a_q || !d.a_pq ||
                        !d.a_gq || !d.a_gq_prev || !d.a_zq || !d.a_H))
        return fail(D2F_EINVAL, "d2f: affine arrays missing");
    if (d.n_ten > 0 && (!d.t_node || !d.t_prv || !d.t_nxt || !d.t_tid || !d.t_stiff || !d.t_L0 ||
                        !d.t_Tcmd || !d.t_state))
        return fail(D2F_EINVAL, "d2f: tendon arrays missing");
    if (!(d.dt > 0.0) || d.iter_max < 0) return fail(D2F_EINVAL, "d2f: dt must be > 0, iter_max >= 0");
    int nt = d.threads ? d.threads : 128;
    if (nt != 32 && nt != 64 && nt != 128 && nt != 256) return fail(D2F_EINVAL, "d2f: threads must be 32, 64, 128 or 256");
    if (!d.inc8) return fail(D2F_EINVAL, "d2f: inc8 (padded node-corner table) is null");
    if (d.line_search) {
        if (!d.xu) return fail(D2F_EINVAL, "d2f: the line search needs xu (2 N + 6 n_aff doubles)");
        if (d.n_backtrack < 0 || !(d.ls_tol >= 0.0)) return fail(D2F_EINVAL, "d2f: n_backtrack >= 0, ls_tol >= 0");
    }
    if (d.n_sp < 0 || (d.n_sp > 0 && (!d.sp_a || !d.sp_b || !d.sp_k || !d.sp_L0 || !d.sp_anchor)))
        return fail(D2F_EINVAL, "d2f: spring arrays missing");
    if (d.n_pe < 0 || d.n_ch < 0 || (d.n_pe > 0 && (d.n_ch <= 0 || !d.pe_a || !d.pe_b || !d.pe_ch || !d.ch_p || !d.ch_ref)))
        return fail(D2F_EINVAL, "d2f: pressure arrays missing");
    if (d.blocks_per_scene != 0 && d.blocks_per_scene != 1 && d.blocks_per_scene != 8 && d.blocks_per_scene != 12 &&
        d.blocks_per_scene != 16 && d.blocks_per_scene != D2F_ALL_SMS)
        return fail(D2F_EINVAL, "d2f: blocks_per_scene must be 0, 1, 8, 12, 16 or D2F_ALL_SMS (-1)");
    if ((d.blocks_per_scene > 1 || d.blocks_per_scene == D2F_ALL_SMS) && d.precision != D2F_MIXED)
        return fail(D2F_EINVAL, "d2f: several blocks per scene run in mixed precision only");
    return D2F_OK;
}

// Blocks per scene: the caller's choice (the next smaller cluster that can be placed when
// it cannot, 1 when none can), else clusters for batches of fewer scenes than SMs whose
// scenes average at least 16384 nodes (a block per scene would leave most SMs idle and each
// scene latency-bound): 16, 12 or 8 blocks, whichever finishes the batch first, taking a
// scene's time on 16 / 12 / 8 blocks as 1 / 1.15 / 1.3 (measured on a 0.26M-node slab) and
// counting the waves of scenes the clusters that fit at once need.
static int blocks_per_scene(const d2f_scene_desc &d, int nsm, int smem) {
    int want = d.blocks_per_scene;
    if (want == 1) return 1;
    if (want == D2F_ALL_SMS) {  // every SM on one scene, when the device and the scratch allow it
        if (nsm <= d2f::grid_max_blocks() && d2f::grid_blocks_mixed(smem) >= nsm)
            return D2F_ALL_SMS;
        want = 0;  // else the library's choice
    }
    if (want == 0 && (d.precision != D2F_MIXED || d.n_scenes >= nsm || d.N / d.n_scenes < 16384)) return 1;
    const int sizes[3] = {16, 12, 8}, cost[3] = {100, 115, 130};
    int best = 1;
    long best_t = 0;
    for (int k = 0; k < 3; ++k) {
        if (want > 0 && sizes[k] > want) continue;
        const int m = d2f::max_clusters_mixed(sizes[k], smem);
        if (m <= 0) continue;
        if (want > 0) return sizes[k];
        const long t = (long)((d.n_scenes + m - 1) / m) * cost[k];
        if (best == 1 || t < best_t) { best = sizes[k]; best_t = t; }
    }
    return best;
}

// Grid (scene blocks), dynamic shared memory and blocks per scene of a launch on the current
// device.
static int launch_shape(const d2f_scene_desc &d, int *grid, int *smem, int *cs) {
    *smem = d.Ne > 0 ? d.max_nb * (int)sizeof(float2) : 0;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(D2F_ECUDA, "d2f: no CUDA device");
    *cs = blocks_per_scene(d, nsm, *smem);
    if (*cs == D2F_ALL_SMS) {  // one block per SM, all on one scene at a time
        *grid = nsm;
        return D2F_OK;
    }
    if (*cs > 1) {  // persistent clusters, one scene each at a time
        int nc = d2f::max_clusters_mixed(*cs, *smem);
        if (nc > d.n_scenes) nc = d.n_scenes;
        *grid = nc * *cs;
        return D2F_OK;
    }
    int vnt, vminb;
    pick_variant(d2f_default_threads(d), d.blocks_per_sm, &vnt, &vminb);
    const int occ = occupancy(d, *smem, vnt, vminb);
    const int bps = d.blocks_per_sm > 0 ? (d.blocks_per_sm < occ ? d.blocks_per_sm : occ) : occ;
    *grid = nsm * bps;
    if (*grid > d.n_scenes) *grid = d.n_scenes;
    return D2F_OK;
}

static cudaError_t launch(const d2f_scene_desc &d, int grid, int smem, int cs, cudaStream_t st) {
    if (cs == D2F_ALL_SMS) return d2f::launch_mixed_grid(d, grid, smem, st);
    if (cs > 1) return d2f::launch_mixed_cluster(cs, d, grid, smem, st);
    int vnt, vminb;
    pick_variant(d2f_default_threads(d), d.blocks_per_sm, &vnt, &vminb);
    return d.precision == D2F_MIXED ? d2f::launch_mixed(vnt, vminb, d, grid, smem, st)
                                    : d2f::launch_fp64(vnt, vminb, d, grid, smem, st);
}

extern "C" {

int32_t d2f_create(const d2f_scene_desc *desc, d2f_solver **out) {
    g_err[0] = 0;
    if (!desc || !out) return fail(D2F_EINVAL, "d2f_create: null argument");
    int rc = validate(*desc, true);
    if (rc != D2F_OK) return rc;
    d2f_solver *s = new d2f_solver();
    s->d = *desc;
    s->d.threads = d2f_default_threads(*desc);
    rc = launch_shape(s->d, &s->grid, &s->smem, &s->cs);
    if (rc != D2F_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return D2F_OK;
}

int32_t d2f_step(d2f_solver *s, void *stream) {
    if (!s) return fail(D2F_EINVAL, "d2f_step: null handle");
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(s->d.work, 0, 4 * sizeof(int32_t), st) != cudaSuccess)
        return fail(D2F_ECUDA, "d2f_step: cudaMemsetAsync failed");
    cudaError_t e = launch(s->d, s->grid, s->smem, s->cs, st);
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "d2f_step: launch failed: %s", cudaGetErrorString(e));
        return D2F_ECUDA;
    }
    return D2F_OK;
}

int32_t d2f_set_dt(d2f_solver *s, double dt, int32_t iter_max) {
    if (!s) return fail(D2F_EINVAL, "d2f_set_dt: null handle");
    if (!(dt > 0.0) || iter_max < 0) return fail(D2F_EINVAL, "d2f_set_dt: dt must be > 0, iter_max >= 0");
    s->d.dt = dt;
    s->d.iter_max = iter_max;
    return D2F_OK;
}

int32_t d2f_stats(d2f_solver *s, void *stream, int32_t *iters, int32_t *active, int32_t *status) {
    if (!s) return fail(D2F_EINVAL, "d2f_stats: null handle");
    cudaStream_t st = (cudaStream_t)stream;
    size_t n = (size_t)s->d.n_scenes * sizeof(int32_t);
    if ((iters && cudaMemcpyAsync(iters, s->d.iters, n, cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
        (active && cudaMemcpyAsync(active, s->d.active, n, cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
        (status && cudaMemcpyAsync(status, s->d.status, n, cudaMemcpyDeviceToHost, st) != cudaSuccess))
        return fail(D2F_ECUDA, "d2f_stats: copy failed");
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(D2F_ECUDA, "d2f_stats: stream sync failed");
    return D2F_OK;
}

int32_t d2f_destroy(d2f_solver *s) {
    delete s;
    return D2F_OK;
}

int32_t d2f_kernels_per_step(const d2f_solver *s) { return s ? 1 : 0; }

int32_t d2f_energy(d2f_solver *s, double *out, void *stream) {
    g_err[0] = 0;
    if (!s || !out) return fail(D2F_EINVAL, "d2f_energy: null argument");
    if (s->d.precision != D2F_FP64) return fail(D2F_EINVAL, "d2f_energy: the energy read-out runs in FP64 solvers");
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(s->d.work, 0, 4 * sizeof(int32_t), st) != cudaSuccess)
        return fail(D2F_ECUDA, "d2f_energy: cudaMemsetAsync failed");
    d2f_scene_desc d = s->d;
    d.energy_out = out;
    cudaError_t e = launch(d, s->grid, s->smem, 1, st);
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "d2f_energy: launch failed: %s", cudaGetErrorString(e));
        return D2F_ECUDA;
    }
    return D2F_OK;
}

int32_t d2f_launch_shape(const d2f_solver *s, int32_t *blocks, int32_t *threads, int32_t *blocks_per_scene) {
    if (!s) return fail(D2F_EINVAL, "d2f_launch_shape: null handle");
    if (blocks) *blocks = s->grid;
    if (threads) {
        int vnt = d2f::kClusterThreads, vminb = 1;
        if (s->cs == 1) pick_variant(d2f_default_threads(s->d), s->d.blocks_per_sm, &vnt, &vminb);
        *threads = vnt;
    }
    if (blocks_per_scene) *blocks_per_scene = s->cs == D2F_ALL_SMS ? s->grid : s->cs;
    return D2F_OK;
}

}  // extern "C"

// ============================================================================ step without allocation
// Some callers cannot call cudaMalloc: code running inside a host that forbids device
// allocation after start-up (a real-time control loop, a plugin whose host owns every
// device buffer and hands it plain pointers, a process whose memory is already reserved).
// d2f_step_noalloc gives them the same step with no allocation anywhere: the per-triangle
// scratch, the contact-candidate lists, the boundary reference positions and the scene
// queue head come from one file-scope device array instead of caller buffers. Every GPU
// that loads this library holds that array (D2F_NOALLOC_SCRATCH_BYTES) until the process
// exits. The array is shared by every call on a device and keeps the last call's contents;
// the queue head is cleared on each call and everything else is rewritten before it is
// read, so no state carries over. That holds for the contact-candidate lists and their
// reference positions only because both step kernels rebuild the list at the start of
// every step (S.rebuild = 1 in the step setup): a kernel that kept a list from one step to
// the next would read another call's list here. Calls whose work overlaps on the GPU
// (different streams, or different threads) race on it: serialise them. The array's device
// address is looked up once per device, on the first call with that device current; after
// cudaDeviceReset on that device the looked-up address belongs to the old context, so the
// entry point must not be called again in that process.
#include <mutex>

static __device__ __align__(256) unsigned char d2f_noalloc_scratch[D2F_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
void *g_noalloc_base[kMaxDevices];
std::mutex g_noalloc_mu;
inline size_t round256(size_t n) { return (n + 255) & ~(size_t)255; }
}  // namespace

extern "C" int32_t d2f_step_noalloc(const d2f_scene_desc *desc, void *stream) {
    g_err[0] = 0;
    if (!desc) return fail(D2F_EINVAL, "d2f_step_noalloc: null descriptor");
    int rc = validate(*desc, false);
    if (rc != D2F_OK) return rc;
    const d2f_scene_desc &in = *desc;
    const size_t rsz = in.precision == D2F_MIXED ? sizeof(float) : sizeof(double);
    const size_t b_work = round256(4 * sizeof(int32_t));
    const size_t b_escr = round256((size_t)in.T * 12 * rsz);
    const size_t b_ecache = round256((size_t)in.T * 9 * rsz);
    const size_t b_cand = in.Ne > 0 ? round256((size_t)in.cand_total * sizeof(int32_t)) : 0;
    const size_t b_ctr = in.Ne > 0 ? round256((size_t)in.cand_total * 2 * sizeof(double)) : 0;
    const size_t b_xref = in.Ne > 0 ? round256((size_t)in.Nb * 2 * sizeof(double)) : 0;
    const size_t b_mscr = in.precision == D2F_MIXED
                              ? round256(d2f_mixed_scratch_bytes(in.N, in.T, in.Nb, in.n_col, in.n_rig)) : 0;
    const size_t need = b_work + b_escr + b_ecache + b_cand + b_ctr + b_xref + b_mscr;
    if (need > (size_t)D2F_NOALLOC_SCRATCH_BYTES) {
        snprintf(g_err, sizeof g_err,
                 "d2f_step_noalloc: this batch needs %zu bytes of scratch (%d triangles, %d candidate "
                 "slots, %d boundary nodes); the static scratch holds %zu bytes. Use d2f_create/d2f_step "
                 "with caller-allocated scratch for batches this large.",
                 need, in.T, in.cand_total, in.Nb, (size_t)D2F_NOALLOC_SCRATCH_BYTES);
        return D2F_EINVAL;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(D2F_ECUDA, "d2f_step_noalloc: no current CUDA device");
    if (dev < 0 || dev >= kMaxDevices) return fail(D2F_EINVAL, "d2f_step_noalloc: device index out of range");
    void *base = nullptr;
    {
        // set-up, once per device, with that device current: the host-side name of a
        // __device__ array is not its device address; ask the runtime for the address.
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_base[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, d2f_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                snprintf(g_err, sizeof g_err, "d2f_step_noalloc: cudaGetSymbolAddress failed: %s",
                         cudaGetErrorString(e));
                return D2F_ECUDA;
            }
            g_noalloc_base[dev] = p;
        }
        base = g_noalloc_base[dev];
    }
    d2f_scene_desc d = in;
    unsigned char *q = static_cast<unsigned char *>(base);
    d.work = reinterpret_cast<int32_t *>(q); q += b_work;
    d.escr = q; q += b_escr;
    d.ecache = q; q += b_ecache;
    d.cand = in.Ne > 0 ? reinterpret_cast<int32_t *>(q) : nullptr; q += b_cand;
    d.cand_tr = in.Ne > 0 ? reinterpret_cast<double *>(q) : nullptr; q += b_ctr;
    d.xref = in.Ne > 0 ? reinterpret_cast<double *>(q) : nullptr; q += b_xref;
    d.mscr = in.precision == D2F_MIXED ? q : nullptr;
    d.threads = d2f_default_threads(in);
    int grid = 0, smem = 0, cs = 1;
    rc = launch_shape(d, &grid, &smem, &cs);
    if (rc != D2F_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(d.work, 0, 4 * sizeof(int32_t), st) != cudaSuccess)  // the queue head starts at 0
        return fail(D2F_ECUDA, "d2f_step_noalloc: cudaMemsetAsync failed");
    cudaError_t e = launch(d, grid, smem, cs, st);
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "d2f_step_noalloc: launch failed: %s", cudaGetErrorString(e));
        return D2F_ECUDA;
    }
    return D2F_OK;
}
