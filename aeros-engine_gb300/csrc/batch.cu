// batch.cu — the C ABI of include/aeros_batch.h: many solver domains stepped
// by one persistent kernel per lattice step, in CUDA-graph-captured chunks.
//
// Nothing here has a counterpart in the reference, which steps one domain at
// a time (stepLBMCPU, aeros/src/lbm.cpp:907-1709). Each member is an ordinary
// aeros_lbm handle; the batch only builds the tile work-list, launches, and
// keeps the members' host-side bookkeeping (AA parity, statistics, divergence
// reset) exactly as aeros_lbm_step would after the same number of steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/aeros_batch.h"
#include "handle.cuh"

using namespace aeros;

struct aeros_batch {
    int storage = AEROS_STORE_FP16;
    const Launchers* L = nullptr;
    std::vector<aeros_lbm*> members;
    aeros_batch_tuning tune{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int sm_count = 1, occ = 1;
    // device tables
    BatchDomain* d_doms = nullptr;
    int cap_doms = 0;
    BatchWork* d_work = nullptr;
    int cap_work = 0, nwork = 0;
    Partial* d_parts = nullptr;
    long long cap_parts = 0;
    unsigned int* d_done = nullptr;
    BatchCtl* d_ctl = nullptr;
    // pinned staging of what every call uploads
    BatchDomain* h_doms = nullptr;
    int cap_h_doms = 0;
    BatchCtl* h_ctl = nullptr;
    // captured chunk
    bool dirty = true;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    float last_ms = 0.0f;
    long long last_launches = 0;
};

namespace {

void drop_graph(aeros_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_steps = 0;
}

int grid_of(const aeros_batch* b) {
    const int bps = b->tune.blocks_per_sm > 0 ? std::min(b->tune.blocks_per_sm, b->occ) : b->occ;
    return std::max(1, b->sm_count * bps);
}

template <class T>
int grow(T** p, long long need, long long* cap) {
    if (need <= *cap) return AEROS_OK;
    const long long n = std::max<long long>(need, *cap * 2);
    T* q = nullptr;
    if (cudaMalloc((void**)&q, (size_t)n * sizeof(T)) != cudaSuccess)
        return set_error(AEROS_ERR_ALLOC, "batch table of %lld entries", n);
    cudaFree(*p);
    *p = q;
    *cap = n;
    return AEROS_OK;
}

// Tile t of a domain is a shell tile when t % k == 0 and t / k < shell tiles
// (the spreading rule of process_tile).
bool is_shell_tile(const StepArgs& A, int t) {
    const int nsh = A.ntiles - A.ntiles_interior;
    return nsh > 0 && (t % A.shell_stride) == 0 && t / A.shell_stride < nsh;
}

// Work-list and device tables for the current members and tuning.
int rebuild(aeros_batch* b) {
    drop_graph(b);
    const int nd = (int)b->members.size();
    std::vector<StepArgs> args(nd);
    std::vector<int> base(nd);
    long long parts = 0;
    for (int i = 0; i < nd; ++i) {
        base_args(b->members[i], args[i]);
        base[i] = (int)parts;
        parts += args[i].ntiles;
    }
    const int tpi = std::max(1, b->tune.tiles_per_item);
    std::vector<BatchWork> work;
    auto add_runs = [&](int d, bool want_shell, bool any) {
        const StepArgs& A = args[d];
        int t = 0;
        while (t < A.ntiles) {
            if (!any && is_shell_tile(A, t) != want_shell) { ++t; continue; }
            int n = 1;
            if (!(want_shell && !any))   // shell tiles are not adjacent: one per item
                while (n < tpi && t + n < A.ntiles && (any || !is_shell_tile(A, t + n))) ++n;
            work.push_back(BatchWork{d, t, n, 0});
            t += n;
        }
    };
    if (b->tune.shell_first) {
        for (int d = 0; d < nd; ++d) add_runs(d, true, false);
        for (int d = 0; d < nd; ++d) add_runs(d, false, false);
    } else {
        for (int d = 0; d < nd; ++d) add_runs(d, false, true);
    }
    long long cap = b->cap_doms;
    if (int rc = grow(&b->d_doms, std::max(1, nd), &cap)) return rc;
    if (cap != b->cap_doms) {
        cudaFree(b->d_done);
        b->d_done = nullptr;
        if (cudaMalloc((void**)&b->d_done, (size_t)cap * sizeof(unsigned int)) != cudaSuccess)
            return set_error(AEROS_ERR_ALLOC, "batch counters");
        b->cap_doms = (int)cap;
    }
    CUDA_TRY(cudaMemsetAsync(b->d_done, 0, (size_t)b->cap_doms * sizeof(unsigned int), b->stream));
    cap = b->cap_work;
    if (int rc = grow(&b->d_work, std::max<long long>(1, (long long)work.size()), &cap)) return rc;
    b->cap_work = (int)cap;
    if (int rc = grow(&b->d_parts, std::max<long long>(1, parts), &b->cap_parts)) return rc;
    if (!work.empty())
        CUDA_TRY(cudaMemcpyAsync(b->d_work, work.data(), work.size() * sizeof(BatchWork), cudaMemcpyHostToDevice,
                                 b->stream));
    b->nwork = (int)work.size();
    if (nd > b->cap_h_doms) {
        if (b->h_doms) cudaFreeHost(b->h_doms);
        b->h_doms = nullptr;
        b->cap_h_doms = 0;
        if (cudaMallocHost((void**)&b->h_doms, (size_t)nd * sizeof(BatchDomain)) != cudaSuccess)
            return set_error(AEROS_ERR_ALLOC, "pinned batch table");
        b->cap_h_doms = nd;
    }
    for (int i = 0; i < nd; ++i) b->h_doms[i].part_base = base[i];
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->dirty = false;
    return AEROS_OK;
}

BatchArgs batch_args(const aeros_batch* b) {
    BatchArgs B;
    B.doms = b->d_doms;
    B.work = b->d_work;
    B.nwork = b->nwork;
    B.partials = b->d_parts;
    B.done = b->d_done;
    B.ctl = b->d_ctl;
    return B;
}

int capture(aeros_batch* b, int steps) {
    drop_graph(b);
    const BatchArgs B = batch_args(b);
    const int grid = grid_of(b);
    CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < steps && le == cudaSuccess; ++i) le = b->L->batch_step(B, (i & 1) != 0, grid, b->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return set_error(AEROS_ERR_CUDA, "batch graph capture: %s",
                         cudaGetErrorString(le != cudaSuccess ? le : ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        b->graph = nullptr;
        return set_error(AEROS_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(ie));
    }
    b->graph_steps = steps;
    return AEROS_OK;
}

int check_member(const aeros_batch* b, const aeros_lbm* h) {
    if (h->p.storage != b->storage)
        return set_error(AEROS_ERR_INVALID, "domain storage %d differs from the batch's %d", h->p.storage, b->storage);
    if (h->th_on) return set_error(AEROS_ERR_STATE, "domains with the thermal lattice cannot join a batch");
    if (h->next_odd) return set_error(AEROS_ERR_STATE, "domain stands at an odd AA-pattern parity");
    return AEROS_OK;
}

}  // namespace

extern "C" int aeros_batch_create(int storage, aeros_batch** out) {
    if (!out) return set_error(AEROS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (storage < AEROS_STORE_FP32 || storage > AEROS_STORE_BF16)
        return set_error(AEROS_ERR_INVALID, "unknown storage %d", storage);
    aeros_batch* b = new (std::nothrow) aeros_batch();
    if (!b) return set_error(AEROS_ERR_ALLOC, "host allocation failed");
    b->storage = storage;
    b->L = storage == AEROS_STORE_FP32 ? &launchers_fp32()
         : storage == AEROS_STORE_FP16 ? &launchers_fp16() : &launchers_bf16();
    b->tune.blocks_per_sm = 0;
    b->tune.tiles_per_item = 1;
    b->tune.shell_first = 1;
    b->tune.chunk_steps = 20;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_ctl, sizeof(BatchCtl));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_ctl, sizeof(BatchCtl));
    if (e != cudaSuccess) {
        aeros_batch_destroy(b);
        return set_error(AEROS_ERR_CUDA, "batch create: %s", cudaGetErrorString(e));
    }
    b->occ = b->L->batch_occupancy();
    *out = b;
    return AEROS_OK;
}

extern "C" int aeros_batch_destroy(aeros_batch* b) {
    if (!b) return set_error(AEROS_ERR_INVALID, "batch is NULL");
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (aeros_lbm* h : b->members) h->batch = nullptr;
    drop_graph(b);
    cudaFree(b->d_doms);
    cudaFree(b->d_work);
    cudaFree(b->d_parts);
    cudaFree(b->d_done);
    cudaFree(b->d_ctl);
    if (b->h_doms) cudaFreeHost(b->h_doms);
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return AEROS_OK;
}

extern "C" int aeros_batch_add(aeros_batch* b, aeros_lbm* h) {
    if (!b || !h) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (h->batch) return set_error(AEROS_ERR_STATE, "domain is already in a batch");
    if (int rc = finish_batch(h)) return rc;
    if (int rc = check_member(b, h)) return rc;
    b->members.push_back(h);
    h->batch = b;
    b->dirty = true;
    return AEROS_OK;
}

extern "C" int aeros_batch_remove(aeros_batch* b, aeros_lbm* h) {
    if (!b || !h) return set_error(AEROS_ERR_INVALID, "NULL argument");
    auto it = std::find(b->members.begin(), b->members.end(), h);
    if (it == b->members.end()) return set_error(AEROS_ERR_INVALID, "domain is not in this batch");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->members.erase(it);
    h->batch = nullptr;
    b->dirty = true;
    return AEROS_OK;
}

extern "C" int aeros_batch_size(aeros_batch* b, int32_t* n_domains, int64_t* n_cells) {
    if (!b) return set_error(AEROS_ERR_INVALID, "batch is NULL");
    long long cells = 0;
    for (const aeros_lbm* h : b->members) cells += h->ncell;
    if (n_domains) *n_domains = (int32_t)b->members.size();
    if (n_cells) *n_cells = cells;
    return AEROS_OK;
}

extern "C" int aeros_batch_step(aeros_batch* b, int nsteps) {
    if (!b) return set_error(AEROS_ERR_INVALID, "batch is NULL");
    if (nsteps < 0 || (nsteps & 1))
        return set_error(AEROS_ERR_INVALID, "nsteps %d: a batch advances by an even number of steps", nsteps);
    b->last_launches = 0;
    b->last_ms = 0.0f;
    if (nsteps == 0 || b->members.empty()) return AEROS_OK;
    for (aeros_lbm* h : b->members) {
        if (int rc = finish_batch(h)) return rc;
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        if (int rc = check_member(b, h)) return rc;
    }
    if (b->dirty)
        if (int rc = rebuild(b)) return rc;
    const int nd = (int)b->members.size();
    for (int i = 0; i < nd; ++i) {
        aeros_lbm* h = b->members[i];
        BatchDomain& D = b->h_doms[i];
        const int base = D.part_base;
        memset(&D, 0, sizeof(D));
        base_args(h, D.A);
        D.u[0] = h->u[0];
        D.u[1] = h->u[1];
        D.out[0] = h->out[0];
        D.out[1] = h->out[1];
        D.ubuf0 = h->ubuf;
        D.outpar0 = h->out_par;
        D.overrides0 = h->overrides_next ? 1 : 0;
        D.les = h->p.use_les ? 1 : 0;
        D.part_base = base;
        h->kexec_before = h->ctl_host->kexec;
    }
    *b->h_ctl = BatchCtl{0u, 0u, 0, nsteps - 1};
    const int chunk = std::max(2, b->tune.chunk_steps & ~1);
    if (!b->graph || b->graph_steps != chunk)
        if (int rc = capture(b, chunk)) return rc;
    CUDA_TRY(cudaMemcpyAsync(b->d_doms, b->h_doms, (size_t)nd * sizeof(BatchDomain), cudaMemcpyHostToDevice,
                             b->stream));
    CUDA_TRY(cudaMemcpyAsync(b->d_ctl, b->h_ctl, sizeof(BatchCtl), cudaMemcpyHostToDevice, b->stream));
    CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
    const int reps = nsteps / chunk, rest = nsteps % chunk;
    for (int r = 0; r < reps; ++r) CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
    const BatchArgs B = batch_args(b);
    for (int i = 0; i < rest; ++i) CUDA_TRY(b->L->batch_step(B, (i & 1) != 0, grid_of(b), b->stream));
    CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
    for (aeros_lbm* h : b->members)
        CUDA_TRY(cudaMemcpyAsync(h->ctl_host, h->ctl, sizeof(Control), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    float ms = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms / (float)nsteps;
    b->last_launches = nsteps;
    int rc_all = AEROS_OK;
    for (aeros_lbm* h : b->members) {
        // the same bookkeeping as nsteps (even) steps of aeros_lbm_step
        h->overrides_next = true;
        h->last_launches = nsteps;
        h->stats_dirty = true;
        h->last_diverged = false;
        if (int rc = finish_batch(h)) rc_all = rc;
    }
    return rc_all;
}

extern "C" int aeros_batch_set_tuning(aeros_batch* b, const aeros_batch_tuning* t) {
    if (!b || !t) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (t->blocks_per_sm < 0 || t->blocks_per_sm > 64) return set_error(AEROS_ERR_INVALID, "blocks_per_sm %d", t->blocks_per_sm);
    if (t->tiles_per_item != 1 && t->tiles_per_item != 2 && t->tiles_per_item != 4 && t->tiles_per_item != 8)
        return set_error(AEROS_ERR_INVALID, "tiles_per_item %d (1, 2, 4 or 8)", t->tiles_per_item);
    if (t->chunk_steps < 2 || (t->chunk_steps & 1) || t->chunk_steps > 10000)
        return set_error(AEROS_ERR_INVALID, "chunk_steps %d (even, 2..10000)", t->chunk_steps);
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->tune = *t;
    b->tune.shell_first = t->shell_first ? 1 : 0;
    b->dirty = true;
    return AEROS_OK;
}

extern "C" int aeros_batch_get_tuning(aeros_batch* b, aeros_batch_tuning* t) {
    if (!b || !t) return set_error(AEROS_ERR_INVALID, "NULL argument");
    *t = b->tune;
    if (t->blocks_per_sm == 0) t->blocks_per_sm = b->occ;
    return AEROS_OK;
}

extern "C" int aeros_batch_autotune(aeros_batch* b, int trial_steps, aeros_batch_tuning* best) {
    if (!b) return set_error(AEROS_ERR_INVALID, "batch is NULL");
    if (trial_steps < 2 || (trial_steps & 1)) return set_error(AEROS_ERR_INVALID, "trial_steps %d (even, >= 2)", trial_steps);
    if (b->members.empty()) return set_error(AEROS_ERR_STATE, "empty batch");
    const aeros_batch_tuning start = b->tune;
    std::vector<aeros_batch_tuning> cand;
    std::vector<int> bps;
    for (int v : {b->occ, b->occ - 1, 2, 1})
        if (v >= 1 && v <= b->occ && std::find(bps.begin(), bps.end(), v) == bps.end()) bps.push_back(v);
    for (int p : bps)
        for (int tpi : {1, 2, 4}) {
            aeros_batch_tuning t = start;
            t.blocks_per_sm = p;
            t.tiles_per_item = tpi;
            t.shell_first = 1;
            t.chunk_steps = std::max(2, std::min(start.chunk_steps, trial_steps));
            cand.push_back(t);
        }
    float best_ms = 1e30f;
    aeros_batch_tuning pick = start;
    auto trial = [&](const aeros_batch_tuning& t) -> int {
        if (int rc = aeros_batch_set_tuning(b, &t)) return rc;
        if (int rc = aeros_batch_step(b, 2)) return rc;   // capture + warm
        if (int rc = aeros_batch_step(b, trial_steps)) return rc;
        if (b->last_ms < best_ms) {
            best_ms = b->last_ms;
            pick = t;
        }
        return AEROS_OK;
    };
    for (const auto& t : cand)
        if (int rc = trial(t)) return rc;
    aeros_batch_tuning alt = pick;
    alt.shell_first = 0;
    if (int rc = trial(alt)) return rc;
    pick.chunk_steps = start.chunk_steps;
    if (int rc = aeros_batch_set_tuning(b, &pick)) return rc;
    if (best) *best = pick;
    return AEROS_OK;
}

extern "C" int aeros_batch_last_step_ms(aeros_batch* b, float* ms) {
    if (!b || !ms) return set_error(AEROS_ERR_INVALID, "NULL argument");
    *ms = b->last_ms;
    return AEROS_OK;
}

extern "C" int aeros_batch_last_launch_count(aeros_batch* b, int64_t* launches) {
    if (!b || !launches) return set_error(AEROS_ERR_INVALID, "NULL argument");
    *launches = b->last_launches;
    return AEROS_OK;
}
