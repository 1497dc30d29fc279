// solver_impl.cuh -- the solver handle behind the C ABI (include/tss.h), shared by
// solver.cu (single scenes and the calls common to every handle) and pool.cu
// (pools and batches of scenes).
//
// Replaces WCSPHSolver + ParticleSystem's device storage (TwoScale2D/WCSPHSolver.cu:
// 2287-3238, TwoScale2D/ParticleSystem.cpp:13-119).  Differences by design:
//  * one device arena per solver, all state resident; no GL interop
//  * the particle counts stay on the device (no per-step readback, 2760-2781);
//    every kernel reads its count from device memory
//  * a whole step is captured once into a CUDA graph and replayed
//  * all handle state is per handle (the reference kept activeID in a function
//    static, 2728)
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/tss.h"
#include "extent.hpp"
#include "grid.cuh"
#include "sph.cuh"

namespace tss {

struct ScaleBufs {
    float2 *pos, *vel, *acc, *npos, *nvel;
    uint8_t *st, *nst;
    int32_t *id, *nid, *map;
    float *dens, *pres, *q, *ndens, *npres;
    float* tr;  // low scale: a split parent's tether radius this step (sorted order)
    uint8_t* cflag;  // low scale: per cell, the step stamp of a cell with an unsplit entry (see ScaleView)
    int16_t* nbr;  // neighbour lists, kMaxNbr x cap (see ScaleView)
    uint8_t* nnbr;
    int cap;       // entries of the sorted arrays
    GridBufs g;
};

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// Bump allocation of many arrays out of one cudaMalloc.
struct Arena {
    std::vector<std::pair<void**, size_t>> items;
    template <class T>
    void add(T** p, size_t count) { items.push_back({reinterpret_cast<void**>(p), al256(sizeof(T) * (count ? count : 1))}); }
    size_t total() const {
        size_t t = 0;
        for (auto& it : items) t += it.second;
        return t;
    }
    void carve(char* base) {
        for (auto& it : items) {
            *it.first = base;
            base += it.second;
        }
    }
};

// One scene as the C ABI describes it.
struct SceneIn {
    const tss_config* cfg;
    int n_low;
    const float* low_pos;
    const float* low_vel;
    float mass_low, mass_high;
    int n_wall;
    const float* wall_pos;
    float mass_wall;
};

// Where an admitted scene lives in a pool.
struct SceneRec {
    bool live = false;
    int64_t sb = 0, n_low = 0;   // low-res slots [sb, sb + n_low); high-res slots 4x
    int64_t cbL = 0, nCL = 0;    // low-res cells [cbL, cbL + nCL), nCL = grid cells + 1
    int64_t cbH = 0, nCH = 0;    // high-res cells
    int64_t wb = 0, nW = 0;      // wall particles
    int64_t high_res = 0;        // high-res list entries reserved
    int64_t admitted_step = 0;   // pool steps issued before the admission
};

bool valid_cfg(const tss_config* cfg);
tss_launch default_launch();  // 256 threads per block, covering grids
Params make_params(const SceneIn& sc);
void scene_runs(const SceneIn& sc, tss_footprint* f);  // unrounded footprint

// Host launchers of small kernels shared by the translation units.
void launch_fill_i32(int32_t* p, int64_t n, int v, cudaStream_t s);
void launch_iota(int32_t* p, int n, cudaStream_t s);
void launch_set_counts(Counters* c, int nL, int nH, cudaStream_t s);
void launch_keys_batched(const float2* pos, const int32_t* id, const int* n_ptr, int cap, const Params* table,
                         const uint16_t* page_scene, int page_shift, int shift, int high, GridBufs g, cudaStream_t s);

}  // namespace tss

struct tss_solver {
    tss_config cfg;
    tss::Params P;               // a single scene's parameters; a pool's capacities
    int nL = 0, capH = 0, slotsL = 0, slotsH = 0, nW = 0;
    int CL = 0, CH = 0;
    bool carry = false;
    bool batched = false;        // a pool or batch of scenes
    char* arena = nullptr;
    size_t arena_bytes = 0;
    tss::ScaleBufs L{}, H{};
    float2* wpos = nullptr;
    int* woff = nullptr;
    uint8_t* wnear = nullptr;  // per low cell (StepView::wnear)
    tss::Counters* cnt = nullptr;
    uint8_t* split_flag = nullptr;
    int32_t* split_ids = nullptr;
    unsigned* split_tile = nullptr;
    int split_ntiles = 1;
    float2* relax_pos = nullptr;
    float2* relax_vel = nullptr;
    cudaStream_t stream = nullptr;
    // step graphs of 1, 2, 4 and 8 steps (bucket b holds 1 << b steps)
    static constexpr int kBuckets = 4;
    cudaGraph_t graph[kBuckets] = {};
    cudaGraphExec_t exec[kBuckets] = {};
    int blocksL = 1, blocksH = 1;           // the non-gather particle kernels
    bool low_full = true;                   // the low-res list is always full (single scenes, batches)
    tss_launch launch{};                    // the gathers' launch shape
    int arith = TSS_ARITH_EXACT;            // the gathers' arithmetic (tss_solver_set_arith)
    int gather_grid[TSS_NUM_GATHERS] = {};  // blocks of each gather for that shape
    bool uploaded[2] = {false, false};  // state replaced since the last step
    bool profile = false;
    cudaEvent_t ev[TSS_NUM_STAGES + 1] = {};
    std::string err;

    // ---- pools and batches ----
    int S = 1;                           // scene table entries
    std::vector<tss::Params> h_table;    // per-scene parameters (host copy)
    tss::Params* d_table = nullptr;
    uint16_t* scL = nullptr;             // scene of each sorted particle
    uint16_t* scH = nullptr;
    uint16_t* page_scene = nullptr;      // [slot pages] scene owning each page of low-res slots
    std::vector<uint16_t> h_page_scene;
    bool reserve_high = false;           // admissions reserve 4 high-res entries per low-res particle
    tss::ExtentSet ex_slots, ex_cellsL, ex_cellsH, ex_walls;
    int64_t high_reserved = 0;
    std::vector<tss::SceneRec> scenes;   // by scene id
    std::vector<int> free_ids;           // unused scene ids (a stack, lowest on top)
    int n_live = 0;
    int64_t live_low = 0;                // low-res particles of the admitted scenes
    int64_t phys_low = 0;                // low-res list entries (retired ones stay until the next build)
    int64_t steps_issued = 0;
    int* usedL = nullptr;                // device ints: cells in use on each scale
    int* usedH = nullptr;
    int* wnum = nullptr;                 // device int: wall count of the scene being admitted
    unsigned* ext_cnt = nullptr;         // device scratch of tss_pool_extract
    tss::GridBufs gW{};                  // wall grid build scratch (per-scene views)
    float2* wraw = nullptr;
    int32_t* wid = nullptr;
    int capW = 0;
    void* render_ws = nullptr;           // tss_solver_render scratch, allocated at its first call
    size_t render_ws_bytes = 0;
    // tss_solver_read_positions_async, set up at its first call: two staging
    // buffers used in turn (positions of both lists and their lengths) and a stream
    // for the copies from them to host memory
    struct ReadBack {
        cudaStream_t stream = nullptr;
        void* mem = nullptr;
        float2* low[2] = {};
        float2* high[2] = {};
        int* counts[2] = {};
        cudaEvent_t staged[2] = {};  // on the caller's stream: the staging copy is done
        cudaEvent_t done[2] = {};    // on rb.stream: the host copy is done (the buffer is free)
        int64_t issued = 0;          // tickets handed out; ticket t used buffer t & 1
        int cap_low = 0, cap_high = 0;  // entries each staging buffer holds per list
    } rb;

    // Ordering of the handle's work on callers' streams.  Every call that enqueues
    // work on a caller's stream first makes that stream wait for the handle's last
    // such work when it went to another stream (enter), and afterwards records
    // work_ev there (leave).  wait_idle() then waits for this handle's work only --
    // that event and the handle's own streams -- instead of the whole device, so
    // other solvers and the host application's streams keep running.  Streams under
    // capture are left as they are (a record there would not be a real event).
    cudaEvent_t work_ev = nullptr;
    cudaStream_t work_stream = nullptr;
    bool work_pending = false;

    static bool capturing(cudaStream_t cs) {
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        return cudaStreamIsCapturing(cs, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
    }
    cudaError_t enter(cudaStream_t cs) {
        if (!work_pending || cs == work_stream || capturing(cs)) return cudaSuccess;
        return cudaStreamWaitEvent(cs, work_ev, 0);
    }
    cudaError_t leave(cudaStream_t cs) {
        if (capturing(cs)) return cudaSuccess;
        cudaError_t e = cudaSuccess;
        if (!work_ev && (e = cudaEventCreateWithFlags(&work_ev, cudaEventDisableTiming)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(work_ev, cs)) != cudaSuccess) return e;
        work_stream = cs;
        work_pending = true;
        return cudaSuccess;
    }
    cudaError_t wait_idle() {
        cudaError_t e = cudaSuccess;
        if (work_pending) e = cudaEventSynchronize(work_ev);
        if (e == cudaSuccess && stream) e = cudaStreamSynchronize(stream);
        if (e == cudaSuccess && rb.stream) e = cudaStreamSynchronize(rb.stream);
        return e;
    }
    // Copies and clears on the handle's own stream; the copies return when done.
    cudaError_t d2h(void* dst, const void* src, size_t bytes) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream);
        return e == cudaSuccess ? cudaStreamSynchronize(stream) : e;
    }
    cudaError_t h2d(void* dst, const void* src, size_t bytes) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
        return e == cudaSuccess ? cudaStreamSynchronize(stream) : e;
    }
    cudaError_t memset0(void* dst, size_t bytes) { return cudaMemsetAsync(dst, 0, bytes, stream); }

    tss_status fail(tss_status st, const std::string& msg) {
        err = msg;
        return st;
    }
    tss_status cuda_fail(cudaError_t e, const char* where) {
        err = std::string(where) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? TSS_OOM : TSS_CUDA_ERROR;
    }

    tss::StepView view() const;
    tss::ReorderArgs reorder_args(tss::ScaleBufs& b, bool high);
    cudaError_t mark(int k, cudaStream_t s);
    cudaError_t enqueue_step(cudaStream_t s);
    cudaError_t prime_keys(cudaStream_t s);
    tss_status apply_launch(const tss_launch& l);  // validates, sizes the grids, drops the graphs

    void drop_graph() {
        for (int b = 0; b < kBuckets; ++b) {
            if (exec[b]) cudaGraphExecDestroy(exec[b]);
            if (graph[b]) cudaGraphDestroy(graph[b]);
            exec[b] = nullptr;
            graph[b] = nullptr;
        }
    }

    // The second branch of a step graph (enqueue_step): a stream that joins the
    // capture, and the events that fork it off and join it back.
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    cudaError_t ensure_side() {
        cudaError_t e = cudaSuccess;
        if (!side) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
        if (e == cudaSuccess && !fork_ev) e = cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming);
        if (e == cudaSuccess && !join_ev) e = cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming);
        return e;
    }

    ~tss_solver() {
        wait_idle();
        drop_graph();
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (join_ev) cudaEventDestroy(join_ev);
        if (side) cudaStreamDestroy(side);
        if (work_ev) cudaEventDestroy(work_ev);
        for (auto& x : ev)
            if (x) cudaEventDestroy(x);
        if (stream) cudaStreamDestroy(stream);
        if (arena) cudaFree(arena);
        if (render_ws) cudaFree(render_ws);
        if (rb.stream) cudaStreamSynchronize(rb.stream);
        for (int b = 0; b < 2; ++b) {
            if (rb.staged[b]) cudaEventDestroy(rb.staged[b]);
            if (rb.done[b]) cudaEventDestroy(rb.done[b]);
        }
        if (rb.stream) cudaStreamDestroy(rb.stream);
        if (rb.mem) cudaFree(rb.mem);
    }
};
