// Batched solves: many factors of uneven sizes and RHS counts swept by ONE
// persistent launch per phase (4 launches for the whole batch, whatever the
// number of systems). No counterpart in the reference.
//
// Every task of every system goes into one merged schedule per phase, sorted
// by its dependency level within its own system (ties: system, then the
// system's own order), so all systems advance together and the ticket order
// stays topological for each of them. The row sweeps' schedule is a
// wavefront over groups of systems (gbchol_batch_options): consecutive
// systems whose work arrays fit a budget form a group, and group g's tasks
// are keyed `skew` levels after group g - 1's, so the x values a leaf row
// gathers were written a few levels earlier by its own group and are still
// in L2. Measured on the 256-system benchmark batch (GB300, FP32, one solve
// without the graph): 19.5 ms with one group; groups one after another
// (skew 0) are slower (21.6 -> 25.9 / 37.4 / 52.7 ms with 64 / 32 / 16 MB
// groups: each group's dependency chain then runs alone), while a wavefront
// of 8 MB groups and skew 4 takes 16.9 ms, 16.4 ms with the lane mode fitted
// to each system's RHS count. Each task carries its system index;
// the kernels read that system's arrays from a descriptor table. The batch
// owns its scratch (permuted work arrays, row and unit flags, tickets and a
// device-resident epoch), so a bound batch solve is free of host
// synchronisation and can be captured in a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <new>
#include <tuple>
#include <vector>

#include "solver_impl.h"

using namespace gbchol;

struct gbchol_batch_s {
    int device = 0;
    int32_t count = 0;
    bool f32 = true;
    std::vector<gbchol_handle> solvers;
    std::vector<int32_t> plan_gen;   // each solver's plan counter when the batch was built
    std::vector<int32_t> nrhs, nslices;
    std::vector<size_t> tmp_off, pbuf_off, row_off, uflag_off;
    std::vector<RowSys> lo_h, pt_h, up_h;
    std::vector<SnSys> sn_lo_h, sn_up_h;
    DevBuf<RowSys> lo_d, pt_d, up_d;
    DevBuf<SnSys> sn_lo_d, sn_up_d;
    DevBuf<int32_t> lo_tasks, lo_sys, pt_tasks, pt_sys, up_tasks, up_sys;
    DevBuf<int32_t> snlo_sys, snlo_code, snup_sys, snup_code;
    int32_t n_lo = 0, n_pt = 0, n_up = 0, n_snlo = 0, n_snup = 0;
    DevBuf<unsigned char> tmp;
    DevBuf<int32_t> flags, uflags, counters, epoch, status;
    bool bound = false;
    int32_t row_variant = 1;  // RowSweepArgs::batched_variant
    bool up_merge = true;     // leaf rows sum their top-row terms in the upper leaf sweep (no pass launch)
};

namespace {

// Merges per-system task lists by (group, key, system, position), or with
// skew > 0 by (key + skew * group, system, position): group g then starts
// skew levels after group g - 1 (a wavefront over the groups).
void merge_tasks(const std::vector<const std::vector<int32_t>*>& tasks,
                 const std::vector<const std::vector<int32_t>*>& keys, const std::vector<int32_t>& group,
                 int32_t skew, std::vector<int32_t>& out_task, std::vector<int32_t>& out_sys) {
    std::vector<std::tuple<int64_t, int64_t, int32_t, int32_t>> all;
    for (size_t s = 0; s < tasks.size(); ++s)
        for (size_t i = 0; i < tasks[s]->size(); ++i) {
            const int64_t key = keys[s] ? (*keys[s])[i] : 0;
            if (skew > 0) all.emplace_back(0, key + (int64_t)skew * group[s], (int32_t)s, (int32_t)i);
            else all.emplace_back(group[s], key, (int32_t)s, (int32_t)i);
        }
    std::sort(all.begin(), all.end());
    out_task.resize(all.size());
    out_sys.resize(all.size());
    for (size_t k = 0; k < all.size(); ++k) {
        const int32_t s = std::get<2>(all[k]), i = std::get<3>(all[k]);
        out_task[k] = (*tasks[s])[i];
        out_sys[k] = s;
    }
}

// Consecutive systems grouped so that each group's work arrays take at most
// `budget` bytes (a system larger than that is a group of its own).
std::vector<int32_t> l2_groups(const std::vector<size_t>& bytes, size_t budget) {
    std::vector<int32_t> g(bytes.size(), 0);
    int32_t cur = 0;
    size_t used = 0;
    for (size_t s = 0; s < bytes.size(); ++s) {
        if (used > 0 && used + bytes[s] > budget) {
            ++cur;
            used = 0;
        }
        g[s] = cur;
        used += bytes[s];
    }
    return g;
}

}  // namespace

extern "C" {

int gbchol_batch_create(int32_t count, const gbchol_handle* solvers, const int32_t* nrhs,
                        int32_t precision, gbchol_batch* out) {
    gbchol_batch_options o;
    o.group_bytes = (int64_t)8 << 20;
    o.skew = 4;
    o.row_variant = 2;
    if (const char* env = std::getenv("GBCHOL_BATCH_GROUP_MB")) o.group_bytes = (int64_t)std::atol(env) << 20;
    if (const char* env = std::getenv("GBCHOL_BATCH_SKEW")) o.skew = std::atoi(env);
    if (const char* env = std::getenv("GBCHOL_BATCH_ROW_VARIANT")) o.row_variant = std::atoi(env);
    return gbchol_batch_create_ex(count, solvers, nrhs, precision, &o, out);
}

int gbchol_batch_create_ex(int32_t count, const gbchol_handle* solvers, const int32_t* nrhs,
                           int32_t precision, const gbchol_batch_options* options, gbchol_batch* out) {
    if (!out) return fail(GBCHOL_EINVAL, "out must not be NULL.");
    if (!options) return fail(GBCHOL_EINVAL, "options must not be NULL.");
    if (options->skew < 0 || (options->row_variant != 1 && options->row_variant != 2))
        return fail(GBCHOL_EINVAL, "Batch options: skew must be >= 0 and row_variant 1 or 2.");
    *out = nullptr;
    if (count < 1 || !solvers || !nrhs) return fail(GBCHOL_EINVAL, "A batch needs at least one solver.");
    if (precision != 0 && precision != 1) return fail(GBCHOL_EINVAL, "precision must be 0 or 1.");
    const bool f32 = precision == 0;
    const int dev = solvers[0] ? solvers[0]->device : 0;
    for (int32_t s = 0; s < count; ++s) {
        const gbchol_solver* h = solvers[s];
        if (!h) return fail(GBCHOL_EINVAL, "Null solver in batch.");
        if (h->device != dev) return fail(GBCHOL_EINVAL, "All solvers of a batch must be on one device.");
        if (!(h->store & (f32 ? GBCHOL_STORE_F32 : GBCHOL_STORE_F64)))
            return fail(GBCHOL_ESTATE, "A solver of the batch keeps no factor of this precision.");
        if (nrhs[s] < 1 || nrhs[s] > GBCHOL_MAX_RHS)
            return fail(GBCHOL_EINVAL, "The number of RHS should be less than 128.");
    }
    DeviceGuard g(dev);
    std::unique_ptr<gbchol_batch_s> b(new (std::nothrow) gbchol_batch_s());
    if (!b) return fail(GBCHOL_ENOMEM, "Out of host memory.");
    b->device = dev;
    b->count = count;
    b->f32 = f32;
    b->solvers.assign(solvers, solvers + count);
    for (int32_t s = 0; s < count; ++s) b->plan_gen.push_back(solvers[s]->plan_gen);
    b->nrhs.assign(nrhs, nrhs + count);
    const size_t es = f32 ? sizeof(float) : sizeof(double);
    size_t tmp_total = 0, rows_total = 0, uflags_total = 0;
    std::vector<int32_t> flags_init;
    for (int32_t s = 0; s < count; ++s) {
        const gbchol_solver* h = solvers[s];
        // the batched supernodal kernel uses the wide RHS slice for every
        // system: 32 columns (FP32) or 16 (FP64)
        const int32_t kw = f32 ? 32 : 16;
        b->nslices.push_back((nrhs[s] + kw - 1) / kw);
        b->tmp_off.push_back(tmp_total);
        tmp_total += (size_t)h->n * nrhs[s] * es;
        tmp_total = (tmp_total + 255) / 256 * 256;
        b->pbuf_off.push_back(tmp_total);
        tmp_total += sn_pbuf_bytes((int)h->plan.parts.size(), nrhs[s], !f32, true);
        tmp_total = (tmp_total + 255) / 256 * 256;
        b->row_off.push_back(rows_total);
        rows_total += (size_t)h->n;
        flags_init.insert(flags_init.end(), h->flags_init.begin(), h->flags_init.end());
        b->uflag_off.push_back(uflags_total);
        uflags_total += (h->plan.units.size() + h->plan.parts.size()) * (size_t)b->nslices.back();
    }
    CUDA_TRY(b->tmp.alloc(std::max<size_t>(tmp_total, 1)));
    CUDA_TRY(b->flags.upload(flags_init.data(), flags_init.size()));
    CUDA_TRY(b->uflags.alloc(std::max<size_t>(uflags_total, 1)));
    CUDA_TRY(cudaMemset(b->uflags.p, 0, sizeof(int32_t) * b->uflags.count));
    CUDA_TRY(b->counters.alloc(10));
    CUDA_TRY(cudaMemset(b->counters.p, 0, sizeof(int32_t) * 10));
    CUDA_TRY(b->status.alloc(1));
    CUDA_TRY(cudaMemset(b->status.p, 0, sizeof(int32_t)));
    {
        const int32_t one = 1;
        CUDA_TRY(b->epoch.upload(&one, 1));
    }
    // merged schedules of the row sweeps: groups of systems in a wavefront
    std::vector<size_t> xbytes;
    for (int32_t s = 0; s < count; ++s) xbytes.push_back((size_t)solvers[s]->n * nrhs[s] * es);
    const size_t budget = options->group_bytes > 0 ? (size_t)options->group_bytes : SIZE_MAX;
    const int32_t skew = options->skew;
    b->row_variant = options->row_variant;
    if (const char* env = std::getenv("GBCHOL_UP_MERGE")) b->up_merge = std::atoi(env) != 0;
    const std::vector<int32_t> grp = l2_groups(xbytes, budget), one(count, 0);
    std::vector<const std::vector<int32_t>*> tl, kl;
    std::vector<int32_t> t, sy;
    for (auto* h : b->solvers) { tl.push_back(&h->plan.lo_tasks); kl.push_back(&h->plan.lo_task_key); }
    merge_tasks(tl, kl, grp, skew, t, sy);
    b->n_lo = (int32_t)t.size();
    CUDA_TRY(b->lo_tasks.upload(t.data(), t.size()));
    CUDA_TRY(b->lo_sys.upload(sy.data(), sy.size()));
    tl.clear(); kl.clear();
    for (auto* h : b->solvers) { tl.push_back(&h->plan.upt_tasks); kl.push_back(nullptr); }
    merge_tasks(tl, kl, one, 0, t, sy);
    b->n_pt = (int32_t)t.size();
    CUDA_TRY(b->pt_tasks.upload(t.data(), t.size()));
    CUDA_TRY(b->pt_sys.upload(sy.data(), sy.size()));
    tl.clear(); kl.clear();
    for (auto* h : b->solvers) { tl.push_back(&h->plan.up_tasks); kl.push_back(&h->plan.up_task_key); }
    merge_tasks(tl, kl, grp, skew, t, sy);
    b->n_up = (int32_t)t.size();
    CUDA_TRY(b->up_tasks.upload(t.data(), t.size()));
    CUDA_TRY(b->up_sys.upload(sy.data(), sy.size()));
    for (int lower = 1; lower >= 0; --lower) {
        std::vector<std::tuple<int32_t, int32_t, int32_t, int32_t>> items;
        for (int32_t s = 0; s < count; ++s) {
            // items in the system's own order (units, and in the lower sweep
            // partial sums ~p), keyed by level then that position
            const SolvePlan& P = b->solvers[s]->plan;
            const std::vector<int32_t>& order = lower ? P.unit_order_lo : P.unit_order_up;
            for (int32_t k = 0; k < (int32_t)order.size(); ++k) {
                const int32_t it = order[k];
                const int32_t lev = it >= 0 ? (lower ? P.unit_level_lo[it] : P.unit_level_up[it])
                                            : P.part_level_lo[~it];
                for (int32_t sl = 0; sl < b->nslices[s]; ++sl) items.emplace_back(lev, s, k, sl);
            }
        }
        std::sort(items.begin(), items.end());
        std::vector<int32_t> isys(items.size()), icode(items.size());
        for (size_t k = 0; k < items.size(); ++k) {
            const int32_t s = std::get<1>(items[k]);
            const SolvePlan& P = b->solvers[s]->plan;
            const int32_t it = (lower ? P.unit_order_lo : P.unit_order_up)[std::get<2>(items[k])];
            isys[k] = s;
            icode[k] = sn_item_code(it, std::get<3>(items[k]));
        }
        if (lower) {
            b->n_snlo = (int32_t)items.size();
            CUDA_TRY(b->snlo_sys.upload(isys.data(), isys.size()));
            CUDA_TRY(b->snlo_code.upload(icode.data(), icode.size()));
        } else {
            b->n_snup = (int32_t)items.size();
            CUDA_TRY(b->snup_sys.upload(isys.data(), isys.size()));
            CUDA_TRY(b->snup_code.upload(icode.data(), icode.size()));
        }
    }
    // descriptors (b/x pointers are bound by gbchol_batch_set_io)
    for (int32_t s = 0; s < count; ++s) {
        gbchol_solver* h = b->solvers[s];
        RowSys base;
        base.perm = h->perm.p;
        base.tmp = b->tmp.p + b->tmp_off[s];
        base.flags = b->flags.p + b->row_off[s];
        base.nrhs = nrhs[s];
        RowSys lo = base, pt = base, up = base;
        lo.rowptr = h->lo_rowptr.p;
        lo.cols = h->lo_cols.p;
        lo.vals = f32 ? (const void*)h->lo_v32.p : (const void*)h->lo_v64.p;
        pt.rowptr = h->upt_rowptr.p;
        pt.cols = h->upt_cols.p;
        pt.vals = f32 ? (const void*)h->upt_v32.p : (const void*)h->upt_v64.p;
        up.rowptr = h->up_rowptr.p;
        up.cols = h->up_cols.p;
        up.vals = f32 ? (const void*)h->up_v32.p : (const void*)h->up_v64.p;
        if (b->up_merge) {
            up.nw_rowptr = pt.rowptr;
            up.nw_cols = pt.cols;
            up.nw_vals = pt.vals;
        }
        b->lo_h.push_back(lo);
        b->pt_h.push_back(pt);
        b->up_h.push_back(up);
        SnSys sn;
        sn.units = h->units.p;
        sn.contribs = h->contribs.p;
        sn.sn_rows = h->sn_rows.p;
        sn.panels = f32 ? (const void*)h->pan32.p : (const void*)h->pan64.p;
        sn.dinv = f32 ? (const void*)h->dinv32.p : (const void*)h->dinv64.p;
        sn.perm = h->perm.p;
        sn.tmp = base.tmp;
        sn.uflags = b->uflags.p + b->uflag_off[s];
        sn.unit_of_row = h->unit_of_row.p;
        sn.parts = h->parts.p;
        sn.pbuf = b->tmp.p + b->pbuf_off[s];
        sn.n_units = (int)h->plan.units.size();
        sn.nrhs = nrhs[s];
        sn.nslices = b->nslices[s];
        b->sn_lo_h.push_back(sn);
        b->sn_up_h.push_back(sn);
    }
    *out = b.release();
    return GBCHOL_OK;
}

int gbchol_batch_set_io(gbchol_batch b, const void* const* bs, void* const* xs) {
    if (!b || !bs || !xs) return fail(GBCHOL_EINVAL, "Null argument.");
    DeviceGuard g(b->device);
    for (int32_t s = 0; s < b->count; ++s) {
        if (!bs[s] || !xs[s]) return fail(GBCHOL_EINVAL, "Null b or x in batch.");
        b->lo_h[s].in = bs[s];
        b->pt_h[s].out = xs[s];
        b->up_h[s].out = xs[s];
        b->sn_up_h[s].out = xs[s];
    }
    CUDA_TRY(b->lo_d.upload(b->lo_h.data(), b->lo_h.size()));
    CUDA_TRY(b->pt_d.upload(b->pt_h.data(), b->pt_h.size()));
    CUDA_TRY(b->up_d.upload(b->up_h.data(), b->up_h.size()));
    CUDA_TRY(b->sn_lo_d.upload(b->sn_lo_h.data(), b->sn_lo_h.size()));
    CUDA_TRY(b->sn_up_d.upload(b->sn_up_h.data(), b->sn_up_h.size()));
    b->bound = true;
    return GBCHOL_OK;
}

int gbchol_batch_solve(gbchol_batch b, void* stream) {
    if (!b) return fail(GBCHOL_EINVAL, "Null batch.");
    for (int32_t s = 0; s < b->count; ++s)
        if (b->solvers[s]->plan_gen != b->plan_gen[s])
            return fail(GBCHOL_ESTATE, "A solver of the batch was replanned after the batch was built; build it again.");
    if (!b->bound) return fail(GBCHOL_ESTATE, "Bind the batch's b and x arrays first (gbchol_batch_set_io).");
    DeviceGuard g(b->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const SweepIO io = b->f32 ? SweepIO::F32 : SweepIO::F64;
    int32_t maxr = 0;
    for (int32_t r : b->nrhs) maxr = std::max(maxr, r);
    RowSweepArgs ra;
    ra.status = b->status.p;
    ra.epoch = b->epoch.p;
    ra.chunk = row_chunk();
    ra.max_nrhs = maxr;
    ra.batched_variant = b->row_variant;
    RowSweepArgs lo = ra;
    lo.sys = b->lo_d.p;
    lo.tasks = b->lo_tasks.p;
    lo.task_sys = b->lo_sys.p;
    lo.ntasks = b->n_lo;
    lo.counters = b->counters.p;
    CUDA_TRY(launch_row_sweep(lo, true, io, s));
    SnSweepArgs sn;
    sn.wide = 1;
    sn.status = b->status.p;
    sn.epoch = b->epoch.p;
    sn.sys = b->sn_lo_d.p;
    sn.item_sys = b->snlo_sys.p;
    sn.item_code = b->snlo_code.p;
    sn.nitems = b->n_snlo;
    sn.counters = b->counters.p + 2;
    CUDA_TRY(launch_sn_sweep(sn, true, io, s));
    sn.sys = b->sn_up_d.p;
    sn.item_sys = b->snup_sys.p;
    sn.item_code = b->snup_code.p;
    sn.nitems = b->n_snup;
    sn.counters = b->counters.p + 4;
    CUDA_TRY(launch_sn_sweep(sn, false, io, s));
    RowSweepArgs pt = ra;
    pt.sys = b->pt_d.p;
    pt.tasks = b->pt_tasks.p;
    pt.task_sys = b->pt_sys.p;
    pt.ntasks = b->n_pt;
    pt.counters = b->counters.p + 8;
    if (!b->up_merge) CUDA_TRY(launch_row_sweep(pt, false, io, s));
    RowSweepArgs up = ra;
    up.sys = b->up_d.p;
    up.tasks = b->up_tasks.p;
    up.task_sys = b->up_sys.p;
    up.ntasks = b->n_up;
    up.counters = b->counters.p + 6;
    CUDA_TRY(launch_row_sweep(up, false, io, s));
    return GBCHOL_OK;
}

int gbchol_batch_info(gbchol_batch b, int32_t* launches, int64_t* nnz_l, int64_t* rows) {
    if (!b) return fail(GBCHOL_EINVAL, "Null batch.");
    if (launches)
        *launches = (b->n_lo > 0) + (b->n_snlo > 0) + (b->n_snup > 0) + (b->n_pt > 0 && !b->up_merge) + (b->n_up > 0);
    int64_t z = 0, r = 0;
    for (auto* h : b->solvers) {
        z += h->F.nnz();
        r += h->n;
    }
    if (nnz_l) *nnz_l = z;
    if (rows) *rows = r;
    return GBCHOL_OK;
}

int gbchol_batch_check(gbchol_batch b, void* stream) {
    if (!b) return fail(GBCHOL_EINVAL, "Null batch.");
    DeviceGuard g(b->device);
    CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    int32_t st = 0;
    CUDA_TRY(cudaMemcpy(&st, b->status.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (st != 0) {
        CUDA_TRY(cudaMemset(b->status.p, 0, sizeof(int32_t)));
        return fail(GBCHOL_ETIMEOUT, "A device-side wait expired during a batched solve; results are invalid.");
    }
    return GBCHOL_OK;
}

int gbchol_batch_destroy(gbchol_batch b) {
    if (!b) return GBCHOL_OK;
    DeviceGuard g(b->device);
    cudaDeviceSynchronize();
    delete b;
    return GBCHOL_OK;
}

}  // extern "C"
