// Batched uneven instances: many independent Laue and Bragg solves of
// different sizes planned once and replayed as one CUDA graph
// (dyfox_batch_*).  No single DYFOX counterpart: a DYFOX caller issues one
// solve_dislocation (laue/solver.py:34-91) or solve_surface_batch
// (bragg/solver.py:182-379) call per instance.
//
// Laue: after each instance's per-angle set-up, ONE persistent launch of
// the compensated single-precision march.  Its CTAs take (instance, row)
// items from a queue sorted by cost, longest first.  For an item the CTA
// evaluates e^{iH} of the row once (pivot set-up in double, segment terms
// in single, sum and 2 pi reduction in float-float or double) into its own
// global slab, then marches every angle group of the instance through it
// with the same register-resident update as dyfox_laue_solve (cp.async
// staging of the slab rows).  H is evaluated once per voxel and never
// stored beyond one row per resident CTA.
//
// Bragg: after each instance's couplings / symbol set-up, one CTA per
// (instance, deviation parameter, plane) system, the systems of the largest
// planes first; one launch per launch shape present (precision, threads and
// columns per thread as a single solve of the instance would take them, so
// that narrow planes do not run at the shape of the widest).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "bragg.cuh"
#include "laue_march.cuh"

namespace dyfox {

// laue.cu
int laue_check_desc(const dyfox_laue_desc *d);
void laue_active_rows(const dyfox_laue_desc *d, int *row0, int *n_rows);
cudaError_t launch_laue_setup(const dyfox_laue_desc *d, const double *s_dev,
                              Kappa *kappa, float4 *kappa32, double2 *scale,
                              float4 *kpair, cudaStream_t stream);
cudaError_t launch_zero_rows(const dyfox_laue_desc *d, void *out, size_t elem,
                             int row0, int n_rows, cudaStream_t stream);
// bragg.cu
cudaError_t launch_bragg_batch(const BraggArgs *insts, const int2 *systems,
                               int n_sys, int threads, int cpl, bool mixed,
                               size_t smem, cudaStream_t stream);
cudaError_t set_bragg_batch_smem(int cpl, bool mixed, size_t smem,
                                 int threads);
size_t bragg_instance_bytes(const dyfox_bragg_desc *d, int *threads, int *cpl);
size_t bragg_instance_smem(const dyfox_bragg_desc *d);
int bragg_instance_prepare(const dyfox_bragg_desc *d, const double *seg_table,
                           const double *y_dev, const double *s_dev,
                           void *out, double *info, char *ws,
                           cudaStream_t stream, BraggArgs *a);

// Depth steps of e^{iH} evaluated per staging chunk of a row.
constexpr int kBatchKB = 8;

struct LaueInst {
    MarchArgs m;
    int sum64;
};

// Registers per thread the march loop of CPL columns per lane needs (the
// single-call march kernels' counts); the e^{iH} staging phase fits in
// them with little spilling, which keeps more warps resident.
constexpr int batch_regs(int cpl) {
    return cpl <= 5 ? 80 : cpl <= 7 ? 104 : cpl <= 9 ? 128 : 168;
}
constexpr int batch_min_blocks(int cpl, int warps) {
    return 65536 / (32 * warps * batch_regs(cpl)) > 1
               ? 65536 / (32 * warps * batch_regs(cpl)) : 1;
}

// One persistent CTA of WARPS warps per (SM x resident slot); items are
// (instance, row).
template <int CPL, int WARPS>
__global__ void __launch_bounds__(32 * WARPS, batch_min_blocks(CPL, WARPS))
laue_batch_kernel(const LaueInst *__restrict__ insts,
                                  const int2 *__restrict__ items, int n_items,
                                  int *ticket, float2 *slabs,
                                  size_t slab_elems) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ MarchArgs args;
    __shared__ int s_item, s_sum64;
    float2 *slab = slabs + (size_t)blockIdx.x * slab_elems;
    for (;;) {
        if (threadIdx.x == 0) {
            const int it = atomicAdd(ticket, 1);
            s_item = it;
            if (it < n_items) {
                const int2 w = items[it];
                args = insts[w.x].m;
                args.row0 = w.y;
                args.csgrid = slab;
                s_sum64 = insts[w.x].sum64;
            }
        }
        __syncthreads();
        if (s_item >= n_items) return;
        const MarchArgs &a = args;
        const int nsteps = a.Nz - 1;
        if (a.hsrc == HS_CS32) {
            for (int k0 = 0; k0 < nsteps; k0 += kBatchKB) {
                const int kn = nsteps - k0 < kBatchKB ? nsteps - k0 : kBatchKB;
                stage_chunk32(a.segs, a.n_seg, a.Nx, a.Ny, a.dx, a.dz, a.row0,
                              k0, kn, s_sum64 != 0, slab, smem);
            }
            // the slab, written here through the generic proxy, is read by
            // the march's bulk copies (async proxy)
            asm volatile("fence.proxy.async.global;" ::: "memory");
            __syncthreads();
        }
        // staged rows: the march specialised for them at compile time
        for (int g = 0; g < a.n_groups; ++g) {
            if (a.hsrc == HS_CS32)
                march_block<float, CPL, HT_STAGED, true>(a, 0, g, smem);
            else
                march_block<float, CPL, HT_GENERIC, true>(a, 0, g, smem);
            __syncthreads();
        }
    }
}

using BatchKernel = void (*)(const LaueInst *, const int2 *, int, int *,
                             float2 *, size_t);

template <int CPL>
static BatchKernel batch_kernel_w(int warps) {
    switch (warps) {
    case 4: return laue_batch_kernel<CPL, 4>;
    case 8: return laue_batch_kernel<CPL, 8>;
    case 16: return laue_batch_kernel<CPL, 16>;
    default: return nullptr;
    }
}

static BatchKernel batch_kernel_for(int cpl, int warps) {
    switch (cpl) {
    case 5: return batch_kernel_w<5>(warps);
    case 7: return batch_kernel_w<7>(warps);
    case 9: return batch_kernel_w<9>(warps);
    case 11: return batch_kernel_w<11>(warps);
    default: return nullptr;
    }
}

struct LaueB {
    int item;               // index in the caller's items
    int row0, n_rows, WA, A, n_groups;
    size_t off_kappa, off_k32, off_scale;
};

struct BraggB {
    int item;
    bool mixed;
    int group;                           // index into BatchLayout::bgroups
    size_t off_ws, bytes, off_y;
};

// Bragg systems that share one launch shape: precision, threads per CTA and
// columns per thread, as a single solve of each instance would choose them.
struct BraggGroup {
    bool mixed;
    int threads, cpl;
    size_t smem = 0;
    int n_sys = 0;
    size_t off_sys = 0;
};

struct BatchLayout {
    std::vector<LaueB> laue;
    std::vector<BraggB> bragg;
    int cpl = 5, warps = 8, ctas_per_sm = 0, grid = 0;
    size_t smem_laue = 0, slab_elems = 0;
    long n_items = 0;
    std::vector<BraggGroup> bgroups;
    size_t off_linst = 0, off_items = 0, off_ticket = 0, off_slabs = 0,
           off_binst = 0, ws = 0;
};

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

static int pow2_at_least(int v) {
    int p = 1;
    while (p < v) p *= 2;
    return p;
}

static int batch_plan(const dyfox_batch_item *items, int n,
                      const dyfox_batch_opts *opts, BatchLayout *L) {
    if (n < 0 || (n > 0 && !items)) {
        set_error("bad item list (n=%d)", n);
        return DYFOX_EINVAL;
    }
    dyfox_batch_opts o;
    memset(&o, 0, sizeof o);
    if (opts) o = *opts;
    L->cpl = o.laue_cols_per_lane ? o.laue_cols_per_lane : 5;
    L->warps = o.laue_warps ? o.laue_warps : 8;
    if (L->cpl != 5 && L->cpl != 7 && L->cpl != 9 && L->cpl != 11) {
        set_error("laue_cols_per_lane %d is not 5, 7, 9 or 11",
                  o.laue_cols_per_lane);
        return DYFOX_EINVAL;
    }
    if (L->warps != 4 && L->warps != 8 && L->warps != 16) {
        set_error("laue_warps %d is not 4, 8 or 16", o.laue_warps);
        return DYFOX_EINVAL;
    }
    if (o.laue_ctas_per_sm < 0 || (o.flags & ~DYFOX_FLAG_H_FP64)) {
        set_error("bad batch options");
        return DYFOX_EINVAL;
    }
    const int cpl = L->cpl, warps = L->warps;
    size_t off = 0;
    size_t max_slab = 0;
    for (int i = 0; i < n; ++i) {
        const dyfox_batch_item &it = items[i];
        if (it.kind == DYFOX_BATCH_LAUE) {
            const dyfox_laue_desc *d = &it.laue;
            int st = laue_check_desc(d);
            if (st) return st;
            if (d->precision != DYFOX_FP32 || d->shift_px != 1.0 ||
                (d->h_source != DYFOX_H_SEGMENTS &&
                 d->h_source != DYFOX_H_NONE) ||
                (d->flags & ~(unsigned)DYFOX_FLAG_H_FP64) || (d->Nx & 1)) {
                set_error("item %d: batched Laue items are DYFOX_FP32, "
                          "shift_px 1, segments or no dislocation, even Nx, "
                          "flags 0 or DYFOX_FLAG_H_FP64", i);
                return DYFOX_ENOSYS;
            }
            const int wa = pow2_at_least(div_up(d->Nx, 32 * cpl));
            if (wa > warps) {
                set_error("item %d: Nx=%d needs %d warps per angle, above "
                          "laue_warps=%d", i, d->Nx, wa, warps);
                return DYFOX_ENOSYS;
            }
            if (!it.s_dev || !it.out ||
                (d->h_source == DYFOX_H_SEGMENTS && d->n_seg > 0 &&
                 !it.seg_table)) {
                set_error("item %d: NULL s_dev, out or seg_table", i);
                return DYFOX_EINVAL;
            }
            LaueB b;
            b.item = i;
            laue_active_rows(d, &b.row0, &b.n_rows);
            b.WA = wa;
            b.A = warps / wa;
            b.n_groups = div_up(d->n_e, b.A);
            const size_t nk = (size_t)d->n_e * (d->Nz - 1);
            b.off_kappa = off; off = al256(off + nk * sizeof(Kappa));
            b.off_k32 = off; off = al256(off + nk * sizeof(float4));
            b.off_scale = off; off = al256(off + d->n_e * sizeof(double2));
            const bool seg = d->h_source == DYFOX_H_SEGMENTS && d->n_seg > 0;
            if (seg) {
                max_slab = std::max(max_slab, (size_t)(d->Nz - 1) * d->Nx);
                L->smem_laue = std::max(L->smem_laue,
                                        stage_chunk32_smem(d->n_seg, kBatchKB));
            }
            const MarchSmem ms = march_smem<float>(
                cpl, b.WA, b.A, d->Nz, seg ? HS_CS32 : HS_NONE, 0, true,
                seg ? ST_DIRECT : ST_COMPUTE, seg ? 8 : 0);
            L->smem_laue = std::max(L->smem_laue, ms.total);
            L->n_items += b.n_rows;
            L->laue.push_back(b);
        } else if (it.kind == DYFOX_BATCH_BRAGG) {
            const dyfox_bragg_desc *d = &it.bragg;
            int threads = 0, bc = 0;
            const size_t bytes = bragg_instance_bytes(d, &threads, &bc);
            if (!bytes) return DYFOX_EINVAL;
            if (!it.s_dev || !it.out || !it.y_values ||
                (d->n_seg > 0 && !it.seg_table)) {
                set_error("item %d: NULL s_dev, out, y_values or seg_table", i);
                return DYFOX_EINVAL;
            }
            BraggB b;
            b.item = i;
            b.mixed = d->precision == DYFOX_FP32;
            b.off_ws = off; off = al256(off + bytes);
            b.bytes = bytes;
            b.off_y = off; off = al256(off + d->n_y * sizeof(double));
            b.group = -1;
            for (size_t g = 0; g < L->bgroups.size(); ++g) {
                const BraggGroup &G = L->bgroups[g];
                if (G.mixed == b.mixed && G.threads == threads && G.cpl == bc)
                    b.group = (int)g;
            }
            if (b.group < 0) {
                BraggGroup G;
                G.mixed = b.mixed;
                G.threads = threads;
                G.cpl = bc;
                L->bgroups.push_back(G);
                b.group = (int)L->bgroups.size() - 1;
            }
            BraggGroup &G = L->bgroups[b.group];
            G.n_sys += d->n_y * d->n_s;
            G.smem = std::max(G.smem, bragg_instance_smem(d));
            L->bragg.push_back(b);
        } else {
            set_error("item %d: unknown kind %d", i, it.kind);
            return DYFOX_EINVAL;
        }
    }
    if (L->n_items > (1L << 30)) {
        set_error("%ld Laue items, above 2^30", L->n_items);
        return DYFOX_ENOSYS;
    }
    // Laue persistent grid.
    if (L->n_items > 0) {
        int dev = 0, sms = 0, occ = 0, optin = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (!e) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount,
                                           dev);
        if (!e) e = cudaDeviceGetAttribute(
                &optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e) return cuda_status(e, "device query");
        if (L->smem_laue > (size_t)optin) {
            set_error("batched march needs %zu bytes of shared memory, the "
                      "device allows %d", L->smem_laue, optin);
            return DYFOX_ESMEM;
        }
        BatchKernel k = batch_kernel_for(cpl, warps);
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)L->smem_laue);
        if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &occ, k, 32 * warps, L->smem_laue);
        if (e) return cuda_status(e, "occupancy");
        if (occ < 1) {
            set_error("batched march cannot be resident (%d threads, %zu "
                      "bytes of shared memory)", 32 * warps, L->smem_laue);
            return DYFOX_ESMEM;
        }
        L->ctas_per_sm = o.laue_ctas_per_sm ? std::min(o.laue_ctas_per_sm, occ)
                                            : occ;
        L->grid = sms * L->ctas_per_sm;
        L->slab_elems = (max_slab + 1) & ~(size_t)1;   // 16-byte slabs
    }
    L->off_linst = off; off = al256(off + L->laue.size() * sizeof(LaueInst));
    L->off_items = off; off = al256(off + (size_t)L->n_items * sizeof(int2));
    // [0] the item ticket, [1] the march's wait status
    L->off_ticket = off; off = al256(off + 2 * sizeof(int));
    L->off_slabs = off;
    off = al256(off + (size_t)L->grid * L->slab_elems * sizeof(float2));
    L->off_binst = off; off = al256(off + L->bragg.size() * sizeof(BraggArgs));
    for (BraggGroup &G : L->bgroups) {
        G.off_sys = off;
        off = al256(off + (size_t)G.n_sys * sizeof(int2));
    }
    L->ws = off;
    return DYFOX_OK;
}

}  // namespace dyfox

struct dyfox_batch {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
    const int *err = nullptr;   // the march's wait status in the workspace
};

using namespace dyfox;

extern "C" int dyfox_batch_workspace_bytes(const dyfox_batch_item *items,
                                           int n, const dyfox_batch_opts *opts,
                                           size_t *bytes) {
    set_error("");
    if (!bytes) {
        set_error("NULL bytes");
        return DYFOX_EINVAL;
    }
    *bytes = 0;
    BatchLayout L;
    int st = batch_plan(items, n, opts, &L);
    if (st) return st;
    *bytes = L.ws ? L.ws : 256;
    return DYFOX_OK;
}

// Records the batch's work on `s` (capturing); fills the Bragg instances'
// arguments (host) on the way.
static int record_batch(const dyfox_batch_item *items, const BatchLayout &L,
                        char *ws, cudaStream_t s,
                        std::vector<BraggArgs> *bargs) {
    cudaError_t e;
    int st;
    if ((e = cudaMemsetAsync(ws + L.off_ticket, 0, 2 * sizeof(int), s)))
        return cuda_status(e, "ticket reset");
    for (const LaueB &b : L.laue) {
        const dyfox_laue_desc *d = &items[b.item].laue;
        if ((e = launch_zero_rows(d, items[b.item].out, sizeof(float2), b.row0,
                                  b.n_rows, s)))
            return cuda_status(e, "zero_rows");
        if (b.n_rows == 0) continue;
        if ((e = launch_laue_setup(d, items[b.item].s_dev,
                                   (Kappa *)(ws + b.off_kappa),
                                   (float4 *)(ws + b.off_k32),
                                   (double2 *)(ws + b.off_scale), nullptr,
                                   s)))
            return cuda_status(e, "laue_setup");
    }
    for (size_t j = 0; j < L.bragg.size(); ++j) {
        const BraggB &b = L.bragg[j];
        const dyfox_batch_item &it = items[b.item];
        if ((st = bragg_instance_prepare(&it.bragg, it.seg_table,
                                         (const double *)(ws + b.off_y),
                                         it.s_dev, it.out, it.info,
                                         ws + b.off_ws, s, &(*bargs)[j])))
            return st;
    }
    if (L.n_items > 0) {
        BatchKernel k = batch_kernel_for(L.cpl, L.warps);
        k<<<L.grid, 32 * L.warps, L.smem_laue, s>>>(
            (const LaueInst *)(ws + L.off_linst),
            (const int2 *)(ws + L.off_items), (int)L.n_items,
            (int *)(ws + L.off_ticket), (float2 *)(ws + L.off_slabs),
            L.slab_elems);
        count_launch(1);
        if ((e = cudaGetLastError())) return cuda_status(e, "laue_batch");
    }
    // One launch per launch shape (largest systems first within each).
    for (const BraggGroup &G : L.bgroups) {
        if (!G.n_sys) continue;
        if ((e = launch_bragg_batch((const BraggArgs *)(ws + L.off_binst),
                                    (const int2 *)(ws + G.off_sys), G.n_sys,
                                    G.threads, G.cpl, G.mixed, G.smem, s)))
            return cuda_status(e, "bragg_batch");
    }
    return DYFOX_OK;
}

extern "C" int dyfox_batch_create(const dyfox_batch_item *items, int n,
                                  const dyfox_batch_opts *opts,
                                  void *workspace, size_t workspace_bytes,
                                  void *stream_, dyfox_batch **out) {
    set_error("");
    if (!out) {
        set_error("NULL batch handle");
        return DYFOX_EINVAL;
    }
    *out = nullptr;
    BatchLayout L;
    int st = batch_plan(items, n, opts, &L);
    if (st) return st;
    if (workspace_bytes < L.ws || (L.ws && !workspace)) {
        set_error("workspace of %zu bytes, %zu needed", workspace_bytes, L.ws);
        return DYFOX_ENOMEM;
    }
    dyfox_batch_opts o;
    memset(&o, 0, sizeof o);
    if (opts) o = *opts;
    char *ws = (char *)workspace;
    cudaStream_t stream = (cudaStream_t)stream_;
    cudaError_t e;

    // Host tables: Laue instances, the item queue (longest first), the
    // Bragg systems (largest planes first); the Bragg planes' y.
    std::vector<LaueInst> linst(L.laue.size());
    std::vector<std::pair<double, int2>> q;
    q.reserve(L.n_items);
    for (size_t j = 0; j < L.laue.size(); ++j) {
        const LaueB &b = L.laue[j];
        const dyfox_batch_item &it = items[b.item];
        const dyfox_laue_desc *d = &it.laue;
        const bool seg = d->h_source == DYFOX_H_SEGMENTS && d->n_seg > 0;
        MarchArgs &a = linst[j].m;
        memset(&a, 0, sizeof a);
        a.Nx = d->Nx; a.Ny = d->Ny; a.Nz = d->Nz; a.n_e = d->n_e;
        a.WA = b.WA; a.A = b.A; a.ncols = 32 * b.WA * L.cpl;
        a.n_groups = b.n_groups;
        a.row0 = 0; a.n_rows = 1;
        a.dx = d->dx; a.dz = d->dz; a.sheet_hw = d->sheet_hw;
        a.hsrc = seg ? HS_CS32 : HS_NONE;
        a.segs = seg ? it.seg_table : nullptr;
        a.n_seg = seg ? d->n_seg : 0;
        a.vc = volterra_consts(d->nu, d->a_core);
        a.kappa = (const Kappa *)(ws + b.off_kappa);
        a.kappa32 = (const float4 *)(ws + b.off_k32);
        a.scale = (const double2 *)(ws + b.off_scale);
        a.out = it.out;
        a.stage = seg ? ST_DIRECT : ST_COMPUTE;
        a.raw_elem = seg ? 8 : 0;
        a.err = (int *)(ws + L.off_ticket) + 1;
        linst[j].sum64 = (d->flags | o.flags) & DYFOX_FLAG_H_FP64 ? 1 : 0;
        const double nsteps = d->Nz - 1;
        const double cost = nsteps * (3.0 * a.n_seg * d->Nx +
                                      (double)b.n_groups * b.A * a.ncols);
        for (int r = 0; r < b.n_rows; ++r)
            q.push_back({cost, make_int2((int)j, b.row0 + r)});
    }
    std::stable_sort(q.begin(), q.end(),
                     [](const std::pair<double, int2> &x,
                        const std::pair<double, int2> &y) {
                         return x.first > y.first;
                     });
    std::vector<int2> qitems(q.size());
    for (size_t i = 0; i < q.size(); ++i) qitems[i] = q[i].second;
    std::vector<std::vector<std::pair<double, int2>>> sys(L.bgroups.size());
    for (size_t j = 0; j < L.bragg.size(); ++j) {
        const dyfox_bragg_desc *d = &items[L.bragg[j].item].bragg;
        const double cost = (double)d->Nz * d->Nx;
        const int p = L.bragg[j].group;
        for (int k = 0; k < d->n_y * d->n_s; ++k)
            sys[p].push_back({cost, make_int2((int)j, k)});
    }
    for (size_t p = 0; p < sys.size(); ++p)
        std::stable_sort(sys[p].begin(), sys[p].end(),
                         [](const std::pair<double, int2> &x,
                            const std::pair<double, int2> &y) {
                             return x.first > y.first;
                         });

    // Uploads (synchronous: the host tables are freed on return).
    if (!linst.empty() &&
        (e = cudaMemcpyAsync(ws + L.off_linst, linst.data(),
                             linst.size() * sizeof(LaueInst),
                             cudaMemcpyHostToDevice, stream)))
        return cuda_status(e, "batch upload");
    if (!qitems.empty() &&
        (e = cudaMemcpyAsync(ws + L.off_items, qitems.data(),
                             qitems.size() * sizeof(int2),
                             cudaMemcpyHostToDevice, stream)))
        return cuda_status(e, "batch upload");
    for (size_t p = 0; p < sys.size(); ++p) {
        std::vector<int2> v(sys[p].size());
        for (size_t i = 0; i < v.size(); ++i) v[i] = sys[p][i].second;
        if (!v.empty() &&
            (e = cudaMemcpyAsync(ws + L.bgroups[p].off_sys, v.data(),
                                 v.size() * sizeof(int2),
                                 cudaMemcpyHostToDevice, stream)))
            return cuda_status(e, "batch upload");
        if ((e = cudaStreamSynchronize(stream)))
            return cuda_status(e, "batch upload");
    }
    for (const BraggB &b : L.bragg) {
        const dyfox_batch_item &it = items[b.item];
        if ((e = cudaMemcpyAsync(ws + b.off_y, it.y_values,
                                 it.bragg.n_y * sizeof(double),
                                 cudaMemcpyHostToDevice, stream)))
            return cuda_status(e, "batch upload");
    }
    if ((e = cudaStreamSynchronize(stream)))
        return cuda_status(e, "batch upload");
    for (const BraggGroup &G : L.bgroups)
        if (G.n_sys &&
            (e = set_bragg_batch_smem(G.cpl, G.mixed, G.smem, G.threads)))
            return cuda_status(e, "bragg_batch attributes");

    // Capture the graph on a private stream.
    cudaStream_t cs;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)))
        return cuda_status(e, "batch stream");
    dyfox_batch *b = new (std::nothrow) dyfox_batch;
    if (!b) {
        cudaStreamDestroy(cs);
        set_error("out of host memory");
        return DYFOX_ENOMEM;
    }
    const unsigned long long before = launch_count_value();
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e) {
        delete b;
        cudaStreamDestroy(cs);
        return cuda_status(e, "begin capture");
    }
    std::vector<BraggArgs> bargs(L.bragg.size());
    st = record_batch(items, L, ws, cs, &bargs);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    b->kernels = (int)(launch_count_value() - before);
    launch_count_restore(before);
    cudaStreamDestroy(cs);
    if (st || e) {
        if (g) cudaGraphDestroy(g);
        delete b;
        return st ? st : cuda_status(e, "end capture");
    }
    b->graph = g;
    b->err = (const int *)(ws + L.off_ticket) + 1;
    // The Bragg instances' arguments, read by the graph's Bragg launches.
    if (!bargs.empty()) {
        e = cudaMemcpyAsync(ws + L.off_binst, bargs.data(),
                            bargs.size() * sizeof(BraggArgs),
                            cudaMemcpyHostToDevice, stream);
        if (!e) e = cudaStreamSynchronize(stream);
    }
    if (!e) e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e) {
        cudaGraphDestroy(g);
        delete b;
        return cuda_status(e, "graph instantiate");
    }
    *out = b;
    return DYFOX_OK;
}

extern "C" int dyfox_batch_launch(dyfox_batch *b, void *stream) {
    set_error("");
    if (!b || !b->exec) {
        set_error("NULL batch");
        return DYFOX_EINVAL;
    }
    cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
    if (e) return cuda_status(e, "graph launch");
    count_launch((unsigned)b->kernels);
    return DYFOX_OK;
}

extern "C" int dyfox_batch_status(const dyfox_batch *b, void *stream) {
    set_error("");
    if (!b || !b->err) {
        set_error("NULL batch");
        return DYFOX_EINVAL;
    }
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, b->err, sizeof(int),
                                    cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
    if (!e) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e) return cuda_status(e, "batch status");
    if (err) {
        set_error("a staged row's copy into shared memory did not complete "
                  "within its bounded wait; its exit waves read NaN");
        return DYFOX_ETIMEOUT;
    }
    return DYFOX_OK;
}

extern "C" int dyfox_batch_kernel_count(const dyfox_batch *b) {
    return b ? b->kernels : 0;
}

extern "C" int dyfox_batch_destroy(dyfox_batch *b) {
    if (!b) return DYFOX_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    delete b;
    return DYFOX_OK;
}
