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
    long long cap_doms = 0;
    BatchAcc* d_acc = nullptr;
    long long cap_acc = 0;
    BatchWork* d_work = nullptr;
    long long cap_work = 0;
    int nwork = 0, nshell_items = 0;
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

// Work-list and device tables for the current members and tuning. Items are
// runs of 32-cell slices: the shell items of every member (shell launch),
// then the interior items (interior launch).
int rebuild(aeros_batch* b) {
    drop_graph(b);
    const int nd = (int)b->members.size();
    std::vector<BatchWork> work;
    auto runs = [&](int d, int kind, int n, int step) {
        for (int s0 = 0; s0 < n; s0 += step) work.push_back(BatchWork{d, kind, s0, std::min(step, n - s0)});
    };
    for (int d = 0; d < nd; ++d) runs(d, 0, (b->members[d]->n_shell + 31) / 32, 8 * b->tune.shell_tiles_per_item);
    b->nshell_items = (int)work.size();
    for (int d = 0; d < nd; ++d) runs(d, 1, (b->members[d]->n_interior + 31) / 32, 8 * b->tune.tiles_per_item);
    if (int rc = grow(&b->d_doms, std::max(1, nd), &b->cap_doms)) return rc;
    if (int rc = grow(&b->d_acc, std::max(1, nd), &b->cap_acc)) return rc;
    CUDA_TRY(cudaMemsetAsync(b->d_acc, 0, (size_t)b->cap_acc * sizeof(BatchAcc), b->stream));
    if (int rc = grow(&b->d_work, std::max<long long>(1, (long long)work.size()), &b->cap_work)) return rc;
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
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->dirty = false;
    return AEROS_OK;
}

BatchArgs batch_args(const aeros_batch* b, int kind) {
    BatchArgs B;
    B.doms = b->d_doms;
    B.work = b->d_work;
    B.item_begin = kind == 0 ? 0 : b->nshell_items;
    B.item_end = kind == 0 ? b->nshell_items : b->nwork;
    B.acc = b->d_acc;
    B.ctl = b->d_ctl;
    return B;
}

int shell_grid_of(const aeros_batch* b) {
    return std::max(1, std::min(b->nshell_items, b->sm_count * b->occ));
}

// One lattice step: the shell launch (when any member has shell items), then
// the interior launch.
cudaError_t launch_step(const aeros_batch* b, bool odd, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    if (b->nshell_items > 0) e = b->L->batch_step(batch_args(b, 0), odd, 0, shell_grid_of(b), s);
    if (e == cudaSuccess) e = b->L->batch_step(batch_args(b, 1), odd, 1, grid_of(b), s);
    return e;
}

int launches_per_step(const aeros_batch* b) { return b->nshell_items > 0 ? 2 : 1; }

int capture(aeros_batch* b, int steps) {
    drop_graph(b);
    CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < steps && le == cudaSuccess; ++i) le = launch_step(b, (i & 1) != 0, b->stream);
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
    b->tune.shell_tiles_per_item = 1;
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
    cudaFree(b->d_acc);
    cudaFree(b->d_work);
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
        D.nslices = (h->n_shell + 31) / 32 + (h->n_interior + 31) / 32;
        h->kexec_before = h->ctl_host->kexec;
    }
    *b->h_ctl = BatchCtl{{0u, 0u}, {0u, 0u}, 0, nsteps - 1};
    const int chunk = std::max(2, b->tune.chunk_steps & ~1);
    if (!b->graph || b->graph_steps != chunk)
        if (int rc = capture(b, chunk)) return rc;
    CUDA_TRY(cudaMemcpyAsync(b->d_doms, b->h_doms, (size_t)nd * sizeof(BatchDomain), cudaMemcpyHostToDevice,
                             b->stream));
    CUDA_TRY(cudaMemcpyAsync(b->d_ctl, b->h_ctl, sizeof(BatchCtl), cudaMemcpyHostToDevice, b->stream));
    CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
    const int reps = nsteps / chunk, rest = nsteps % chunk;
    for (int r = 0; r < reps; ++r) CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
    for (int i = 0; i < rest; ++i) CUDA_TRY(launch_step(b, (i & 1) != 0, b->stream));
    CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
    for (aeros_lbm* h : b->members)
        CUDA_TRY(cudaMemcpyAsync(h->ctl_host, h->ctl, sizeof(Control), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    float ms = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms / (float)nsteps;
    b->last_launches = (long long)nsteps * launches_per_step(b);
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
    for (int v : {t->tiles_per_item, t->shell_tiles_per_item})
        if (v != 1 && v != 2 && v != 4 && v != 8)
            return set_error(AEROS_ERR_INVALID, "tiles per item %d (1, 2, 4 or 8)", v);
    if (t->chunk_steps < 2 || (t->chunk_steps & 1) || t->chunk_steps > 10000)
        return set_error(AEROS_ERR_INVALID, "chunk_steps %d (even, 2..10000)", t->chunk_steps);
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->tune = *t;
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
            t.shell_tiles_per_item = 1;
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
    for (int stpi : {2, 4}) {
        aeros_batch_tuning alt = pick;
        alt.shell_tiles_per_item = stpi;
        if (int rc = trial(alt)) return rc;
    }
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
