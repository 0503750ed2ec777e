// handle.cuh — the solver handle shared by the C-ABI translation units
// (capi.cu: single domains; batch.cu: many domains in one persistent kernel).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/aeros_lbm.h"
#include "lbm_aux.cuh"

struct aeros_batch;

// Records code + message (thread-local) for aeros_consume_error; returns code.
int set_error(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));

#define CUDA_TRY(expr)                                                                                    \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return set_error(AEROS_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(e_)); \
    } while (0)

// One lattice domain: device buffers, AA-pattern layout state, statistics.
struct aeros_lbm {
    aeros_lbm_params p{};
    int nx = 0, ny = 0, nz = 0, ncell = 0;
    long long qstride = 0;
    const aeros::Launchers* L = nullptr;
    size_t esize = 4;
    // device memory
    void* f = nullptr;
    uint32_t* desc = nullptr;
    int* shell = nullptr;
    unsigned long long* shell_kind = nullptr;
    uint32_t* shell_gth = nullptr;   // odd-step gather / scatter offsets of the shell cells (NULL: resolve)
    uint32_t* shell_sct = nullptr;
    int* zg_src = nullptr;            // zero-gradient outlet sources (NULL: computed on the device)
    // post-processing (allocated on first use)
    float *uxw = nullptr, *uyw = nullptr, *uzw = nullptr, *pressure = nullptr, *vort = nullptr, *qcrit = nullptr;
    float* prev_rho = nullptr;
    float* u_split = nullptr;         // readback scratch: ux, uy, uz planes (allocated on first use)
    void* post_parts = nullptr;
    void* post_out = nullptr;
    unsigned int* post_counter = nullptr;
    long long post_prev_step = -1;
    float post_prev_maxu = 0.0f;
    float post_min[3] = {0.0f, 0.0f, 0.0f}, post_cell[3] = {1.0f, 1.0f, 1.0f};
    std::vector<int> shell_host;
    std::vector<unsigned long long> shell_kind_host;
    float4* u[2] = {nullptr, nullptr};   // velocity (ux, uy, uz, 0), double buffered
    float4* u_alloc[2] = {nullptr, nullptr};   // their allocations: VEL_GUARD cells of slack on both sides
    float *rho = nullptr, *strain = nullptr, *tke = nullptr;
    float* out[2] = {nullptr, nullptr};
    int out_plane = 0;
    void* g = nullptr;
    float* T = nullptr;
    float* T_buoy = nullptr;
    aeros::Partial* partials = nullptr;
    int max_grid = 0;
    aeros::Control* ctl = nullptr;
    aeros::Control* ctl_host = nullptr;   // pinned
    double* force_partials = nullptr;
    double* force_out = nullptr;
    double* force_host = nullptr;     // pinned: the force sums read back (3 doubles) and the area count
    unsigned int* force_counter = nullptr;
    unsigned long long* area_count = nullptr;
    uint64_t dev_bytes = 0;
    // host geometry
    std::vector<uint8_t> mask, wall;
    int n_interior = 0, n_shell = 0, fluid_cells = 1;
    int outlet_mode = 0;
    float feq_in[19] = {0};
    aeros::Shift19 shift{};      // shifted storage: s_q - w_q (zero for FP32)
    float conv = 0.08f;
    // layout state of the AA pattern
    bool next_odd = false;        // next step gathers from neighbours
    bool overrides_next = false;  // next gather applies inlet/outlet overrides
    int out_par = 1;              // side buffer written by the next step
    int ubuf = 0;                 // u[ubuf] holds the latest velocity
    int grid[2][2] = {{0, 0}, {0, 0}};
    // thermal
    bool th_on = false;
    aeros_thermal_params tp{};
    int ylo = 0, yhi = 0;
    float H = 1, tau_t = 0.7f, alpha = 0, glb = 0;
    int th_buoy_mode = 1;
    bool th_stepped = false;
    // stats
    aeros_lbm_stats stats{};
    bool stats_dirty = false;
    long long kexec_before = 0;
    bool last_diverged = false;
    // timing
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    long long last_launches = 0;
    int sm_count = 0;
    int split = 1;                // shell and interior as two launches per step (AEROS_SPLIT=0: one)
    int fused = 1;                // non-thermal: one launch, dynamic warp items (AEROS_FUSED=0: off)
    int shell_blocks_per_sm = 1;  // fused: shell blocks per SM, 0: shell tiles first in the queue (AEROS_SHELL_BLOCKS)
    bool shell_blocks_set = false;   // AEROS_SHELL_BLOCKS given
    int fused_grid[2][2] = {{0, 0}, {0, 0}};   // fused: interior blocks [odd][thermal]
    bool warp = false;            // non-thermal steps through k_lbm_warp where the shape allows (AEROS_WARP=1)
    int warp_grid[2] = {0, 0};    // warp tiles: interior blocks [odd]
    long long last_kernels = 0;   // kernel launches of the last step call
    aeros_batch* batch = nullptr; // batch this domain is a member of
};

// Kernel arguments of the domain's current state (capi.cu).
void base_args(const aeros_lbm* h, aeros::StepArgs& A);
// Per-step arguments of the next step (parity of the double buffers).
aeros::StepVar step_var(const aeros_lbm* h, bool write_obs);
// Completes the last enqueued steps: statistics, divergence reset.
int finish_batch(aeros_lbm* h);
