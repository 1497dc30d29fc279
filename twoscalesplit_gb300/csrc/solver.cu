// solver.cu -- host side of the solver behind the C ABI (include/tss.h): the step
// sequence, single-scene creation and the calls common to every handle.  Pools and
// batches of scenes are in pool.cu; the handle itself is in solver_impl.cuh.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "solver_impl.cuh"

using namespace tss;

StepView tss_solver::view() const {
    StepView v{};
    auto sv = [](const ScaleBufs& b) {
        ScaleView s{};
        s.pos = b.pos;
        s.vel = b.vel;
        s.st = b.st;
        s.id = b.id;
        s.dens = b.dens;
        s.pres = b.pres;
        s.q = b.q;
        s.tr = b.tr;
        s.cflag = b.cflag;
        s.nbr = b.nbr;
        s.nnbr = b.nnbr;
        s.nbr_stride = b.cap;
        s.acc = b.acc;
        s.off = b.g.off;
        s.map = b.map;
        s.npos = b.npos;
        s.nvel = b.nvel;
        s.nst = b.nst;
        s.nid = b.nid;
        s.ndens = b.ndens;
        s.npres = b.npres;
        s.gcount = b.g.count;
        s.gkey = b.g.key;
        s.grank = b.g.rank;
        s.gtile = b.g.tile_sum;
        return s;
    };
    v.L = sv(L);
    v.H = sv(H);
    if (!carry) {
        v.L.ndens = v.L.npres = nullptr;
        v.H.ndens = v.H.npres = nullptr;
    }
    v.wpos = wpos;
    v.woff = woff;
    v.wnear = wnear;
    v.cnt = cnt;
    v.split_flag = split_flag;
    v.split_ids = split_ids;
    v.split_tile = split_tile;
    v.relax_pos = relax_pos;
    v.relax_vel = relax_vel;
    v.nL = nL;
    v.table = d_table;
    v.scL = scL;
    v.scH = scH;
    return v;
}

ReorderArgs tss_solver::reorder_args(ScaleBufs& b, bool high) {
    ReorderArgs a{};
    a.src_pos = b.npos;
    a.src_vel = b.nvel;
    a.src_st = b.nst;
    a.dst_pos = b.pos;
    a.dst_vel = b.vel;
    a.dst_st = b.st;
    a.dst_id = b.id;
    a.slot_map = b.map;
    a.slots = high ? slotsH : slotsL;
    if (carry) {
        a.src_dens = b.ndens;
        a.src_pres = b.npres;
        a.dst_dens = b.dens;
        a.dst_pres = b.pres;
    }
    if (high) a.h_state0 = &cnt->h_state0;
    if (batched) {
        a.dst_sc = high ? scH : scL;
        a.page_scene = page_scene;
        a.page_shift = 8;  // log2(TSS_POOL_SLOT_PAGE)
        a.id_shift = high ? 2 : 0;
    }
    return a;
}

// cudaEventRecordExternal makes the record a node of the captured graph (a plain
// record inside capture only orders streams)
cudaError_t tss_solver::mark(int k, cudaStream_t s) {
    return profile ? cudaEventRecordWithFlags(ev[k], s, cudaEventRecordExternal) : cudaSuccess;
}

// Enqueue one step (the body of AdvanceTS, WCSPHSolver.cu:2726-2810).
cudaError_t tss_solver::enqueue_step(cudaStream_t s) {
    cudaError_t e;
    StepView V = view();
    // the force passes read the neighbour lists their scale's density pass records
    // when that pass runs one particle per thread
    if (launch.per_warp[1]) V.L.nbr = nullptr;
    if (launch.per_warp[0]) V.H.nbr = nullptr;
    // Outside profiling, the two grid builds and the two density passes each run as
    // two branches of the step graph: the low-res one on the side stream beside the
    // high-res one, joined before the first kernel that reads both (and the split
    // compaction beside the high-res force, below).  Neither of a pair reads what
    // the other writes (they share only atomic ORs into the error word), so the
    // results are those of the sequential order; the branches fill each other's
    // partial last waves and the grid builds' launch gaps.  Profiling keeps the
    // sequential order, so that each stage has its own interval.
    const bool branch = !profile && side != nullptr;
    auto fork = [&]() -> cudaError_t {
        cudaError_t e2 = cudaEventRecord(fork_ev, s);
        return e2 == cudaSuccess ? cudaStreamWaitEvent(side, fork_ev, 0) : e2;
    };
    auto join = [&]() -> cudaError_t {
        cudaError_t e2 = cudaEventRecord(join_ev, side);
        return e2 == cudaSuccess ? cudaStreamWaitEvent(s, join_ev, 0) : e2;
    };
    const cudaStream_t sl = branch ? side : s;  // the low-res branch's stream
    if ((e = mark(0, s)) != cudaSuccess) return e;
    // 1. neighbour grids: high then low (updateNeighborGridHigh / updateNeighborGrid);
    //    their key pass ran at the end of the previous step (force kernels, split),
    //    in prime_keys() after the state was set, or in a pool admission
    if (branch && (e = fork()) != cudaSuccess) return e;
    e = grid_sort_enqueue(H.nid, &cnt->cur[1], capH, H.g, reorder_args(H, true), &cnt->err, s);
    if (e != cudaSuccess || (e = mark(1, s)) != cudaSuccess) return e;
    e = grid_sort_enqueue(L.nid, &cnt->cur[0], nL, L.g, reorder_args(L, false), &cnt->err, sl);
    if (e != cudaSuccess || (e = mark(2, s)) != cudaSuccess) return e;
    if (branch && (e = join()) != cudaSuccess) return e;
    // 2. relaxation of last step's children (older snapshot's relaxTransient)
    for (int it = 0; it < P.relax_iters; ++it) {
        launch_k_relax_density(batched, blocksH, 256, s, P, V);
        launch_k_relax_force(batched, blocksH, 256, s, P, V);
        k_relax_apply<<<blocksH, 256, 0, s>>>(P, V);
    }
    if ((e = mark(3, s)) != cudaSuccess) return e;
    // 3. densities, 4. low force + advance + split marks, 5. children, 6. high force
    const bool fast = arith == TSS_ARITH_FAST;
    auto gather = [&](int g, cudaStream_t gs) {
        launch_gather(g, batched, launch.per_warp[g] != 0, fast, gather_grid[g], launch.threads[g], gs, P, V);
    };
    if (branch && (e = fork()) != cudaSuccess) return e;
    gather(0, s);
    if ((e = mark(4, s)) != cudaSuccess) return e;
    gather(1, sl);
    if ((e = mark(5, s)) != cudaSuccess) return e;
    if (branch && (e = join()) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(split_tile, 0, sizeof(unsigned) * split_ntiles, s)) != cudaSuccess) return e;
    gather(2, s);
    if ((e = mark(6, s)) != cudaSuccess) return e;
    // The split compaction appends children past the high-res list that the
    // high-res force walks, and the two share only atomic adds into the next grid's
    // cell counts: outside profiling they run as two branches too.
    if (branch && (e = fork()) != cudaSuccess) return e;
    launch_k_split(batched, std::min(split_ntiles, 8 * sm_count()), kSplitThreads, sl, P, V);
    if ((e = mark(7, s)) != cudaSuccess) return e;
    gather(3, s);
    if (branch && (e = join()) != cudaSuccess) return e;
    k_step_finish<<<1, 32, 0, s>>>(cnt);
    if ((e = mark(8, s)) != cudaSuccess) return e;
    return cudaGetLastError();
}

// Grid of each gather for launch shape l: a covering grid is one block per
// `threads` list entries of capacity (a full low-res list: exactly its particles;
// otherwise at most 4096 threads per SM, striding beyond); a persistent grid is
// one wave of resident blocks.
tss_status tss_solver::apply_launch(const tss_launch& l) {
    for (int g = 0; g < TSS_NUM_GATHERS; ++g) {
        const int t = l.threads[g];
        if (t != 64 && t != 128 && t != 256) return fail(TSS_INVALID_ARG, "threads per block must be 64, 128 or 256");
        if (l.persistent[g] != 0 && l.persistent[g] != 1) return fail(TSS_INVALID_ARG, "persistent must be 0 or 1");
        if (l.per_warp[g] != 0 && l.per_warp[g] != 1) return fail(TSS_INVALID_ARG, "per_warp must be 0 or 1");
    }
    const long long sms = sm_count();
    int grid[TSS_NUM_GATHERS];
    for (int g = 0; g < TSS_NUM_GATHERS; ++g) {
        const int t = l.threads[g];
        const bool low = g == 1 || g == 2;
        const long long lanes = l.per_warp[g] ? 32 : 1;  // threads per particle
        const long long cap = std::max(low ? nL : capH, 1) * lanes;
        const long long cover = (cap + t - 1) / t;
        if (l.persistent[g]) {
            const int occ = gather_occupancy(g, batched, l.per_warp[g] != 0, arith == TSS_ARITH_FAST, t);
            if (occ <= 0) return fail(TSS_CUDA_ERROR, "occupancy query of a gather kernel failed");
            grid[g] = static_cast<int>(sms * occ);
        } else if (low && low_full) {
            grid[g] = static_cast<int>(std::min<long long>(cover, 0x7fffffffLL));
        } else {
            grid[g] = static_cast<int>(std::min(cover, sms * 4096 / t));
        }
    }
    launch = l;
    for (int g = 0; g < TSS_NUM_GATHERS; ++g) gather_grid[g] = grid[g];
    drop_graph();
    return TSS_OK;
}

tss_launch tss::default_launch() {
    tss_launch l{};
    for (int g = 0; g < TSS_NUM_GATHERS; ++g) {
        l.threads[g] = 256;
        l.persistent[g] = 0;
        l.per_warp[g] = 0;
    }
    return l;
}

// Key pass of both grids for the current list arrays (after create or upload).
cudaError_t tss_solver::prime_keys(cudaStream_t s) {
    cudaError_t e;
    for (ScaleBufs* b : {&L, &H}) {
        if ((e = cudaMemsetAsync(b->g.count, 0, sizeof(unsigned) * static_cast<size_t>(b->g.ncells), s)) !=
            cudaSuccess)
            return e;
        if ((e = cudaMemsetAsync(b->g.tile_sum, 0, sizeof(unsigned) * b->g.ntiles, s)) != cudaSuccess) return e;
    }
    if (batched) {
        launch_keys_batched(H.npos, H.nid, &cnt->cur[1], capH, d_table, page_scene, 8, 2, 1, H.g, s);
        launch_keys_batched(L.npos, L.nid, &cnt->cur[0], nL, d_table, page_scene, 8, 0, 0, L.g, s);
        return cudaGetLastError();
    }
    e = grid_keys_enqueue(H.npos, &cnt->cur[1], capH, P.ox, P.oy, P.rh, P.dimH[0], P.dimH[1], H.g, s);
    if (e != cudaSuccess) return e;
    return grid_keys_enqueue(L.npos, &cnt->cur[0], nL, P.ox, P.oy, P.r, P.dimL[0], P.dimL[1], L.g, s);
}

namespace {

__global__ void k_iota(int32_t* p, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}
__global__ void k_fill_i32(int32_t* p, int64_t n, int v) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        p[i] = v;
}
__global__ void k_set_counts(Counters* c, int nL, int nH) {
    c->cur[0] = c->next[0] = nL;
    c->cur[1] = c->next[1] = nH;
    c->h_state0 = 0;
    c->n_drop = c->dropped = 0;
}
__global__ void k_set_fresh(Counters* c, int n) { c->n_fresh = n; }

// Positions of both lists and their lengths n[2] into caller memory (page-locked
// host memory for tss_solver_read_positions; a staging buffer and then host memory
// for the asynchronous form).
__global__ void k_read_positions(const float2* __restrict__ lowp, const float2* __restrict__ highp,
                                 const int* __restrict__ n, float2* out_low, int cap_low, float2* out_high,
                                 int cap_high, int* counts) {
    const int nl = n[0], nh = n[1];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counts[0] = nl;
        counts[1] = nh;
    }
    const int ml = min(nl, cap_low), mh = min(nh, cap_high);
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ml; i += stride) out_low[i] = lowp[i];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < mh; i += stride) out_high[i] = highp[i];
}

// Key pass of a pool's list: each entry's parameters come from the scene owning
// its slot's page.
__global__ void k_keys_batched(const float2* __restrict__ pos, const int32_t* __restrict__ id,
                               const int* __restrict__ n_ptr, const Params* __restrict__ table,
                               const uint16_t* __restrict__ page_scene, int page_shift, int shift, int high,
                               GridBufs g) {
    const int n = *n_ptr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Params& P = table[page_scene[(id[i] >> shift) >> page_shift]];
        const int c = high ? P.cbH + cell_hash(pos[i], P.ox, P.oy, P.rh, P.dimH[0], P.dimH[1])
                           : P.cbL + cell_hash(pos[i], P.ox, P.oy, P.r, P.dimL[0], P.dimL[1]);
        grid_key(g.count, g.key, g.rank, g.tile_sum, i, c);
    }
}

// Largest x with sqrtf(x) <= r (le) or sqrtf(x) < r (lt).  IEEE square root is
// correctly rounded and monotone on the host and (with -prec-sqrt=true) on the
// device, so `x <= T` decides a cutoff test exactly without taking the root.
float sq_cutoff(float r, bool inclusive) {
    auto ok = [&](float x) { return inclusive ? std::sqrt(x) <= r : std::sqrt(x) < r; };
    float x = r * r;
    while (ok(std::nextafter(x, INFINITY))) x = std::nextafter(x, INFINITY);
    while (x > 0.0f && !ok(x)) x = std::nextafter(x, 0.0f);
    return x;
}

bool finite_cfg(const tss_config* c) {
    const float v[] = {c->domain_origin[0], c->domain_origin[1], c->domain_end[0], c->domain_end[1], c->r_low,
                       c->r_high, c->rest_density, c->tait_b, c->speed_sound, c->alpha, c->tension, c->dt,
                       c->gravity, c->relax_dt_div, c->roi_velocity[0], c->roi_velocity[1]};
    for (float x : v)
        if (!std::isfinite(x)) return false;
    return true;
}

}  // namespace

namespace tss {

void launch_fill_i32(int32_t* p, int64_t n, int v, cudaStream_t s) {
    if (n <= 0) return;
    const int b = particle_blocks(n < (1LL << 30) ? static_cast<int>(n) : (1 << 30), 256);
    k_fill_i32<<<b, 256, 0, s>>>(p, n, v);
}
void launch_iota(int32_t* p, int n, cudaStream_t s) {
    if (n > 0) k_iota<<<particle_blocks(n, 256), 256, 0, s>>>(p, n);
}
void launch_set_counts(Counters* c, int nL, int nH, cudaStream_t s) { k_set_counts<<<1, 1, 0, s>>>(c, nL, nH); }
void launch_keys_batched(const float2* pos, const int32_t* id, const int* n_ptr, int cap, const Params* table,
                         const uint16_t* page_scene, int page_shift, int shift, int high, GridBufs g, cudaStream_t s) {
    k_keys_batched<<<particle_blocks(cap > 0 ? cap : 1, 256), 256, 0, s>>>(pos, id, n_ptr, table, page_scene,
                                                                           page_shift, shift, high, g);
}

// Support radii in [2^-40, 2^40] (about 1e-12 to 1e12): the range in which the
// pair kernels' division by a radius (div_const) is exact.  The reference's own
// gradient coefficient -120/(14 pi r^3) overflows FP32 below about 1e-13.
bool in_radius_range(float r) { return r >= 0x1p-40f && r <= 0x1p40f; }

bool valid_cfg(const tss_config* cfg) {
    if (!cfg || !finite_cfg(cfg) || cfg->dims_low[0] <= 0 || cfg->dims_low[1] <= 0 || cfg->dims_high[0] <= 0 ||
        cfg->dims_high[1] <= 0 || !in_radius_range(cfg->r_low) || !in_radius_range(cfg->r_high) || cfg->relax_iters < 0 ||
        cfg->relax_iters > 64 || !(cfg->relax_dt_div > 0))
        return false;
    return static_cast<long long>(cfg->dims_low[0]) * cfg->dims_low[1] < (1LL << 31) - 2 &&
           static_cast<long long>(cfg->dims_high[0]) * cfg->dims_high[1] < (1LL << 31) - 2;
}

// Per-scene constants, as Bind() derives them (WCSPHSolver.cu:2537-2611).
Params make_params(const SceneIn& sc) {
    const tss_config* cfg = sc.cfg;
    Params P{};
    P.ox = cfg->domain_origin[0];
    P.oy = cfg->domain_origin[1];
    P.dimL[0] = cfg->dims_low[0];
    P.dimL[1] = cfg->dims_low[1];
    P.dimH[0] = cfg->dims_high[0];
    P.dimH[1] = cfg->dims_high[1];
    P.r = cfg->r_low;
    P.rh = cfg->r_high;
    P.rho0 = cfg->rest_density;
    P.B = cfg->tait_b;
    P.cs = cfg->speed_sound;
    P.alpha = cfg->alpha;
    P.sigma = cfg->tension;
    P.dt = cfg->dt;
    P.g = cfg->gravity;
    const double r = cfg->r_low, rh = cfg->r_high;  // Bind(), 2559-2590
    P.CL = static_cast<float>(20.0 / (14.0 * kPi * r * r));
    P.GL = static_cast<float>(-120.0 / (14.0 * kPi * r * r * r));
    P.CH = static_cast<float>(20.0 / (14.0 * kPi * rh * rh));
    P.GH = static_cast<float>(-120.0 / (14.0 * kPi * rh * rh * rh));
    P.mL = sc.mass_low;
    P.mH = sc.mass_high;
    P.mB = sc.mass_wall;
    P.cBL = sc.mass_wall / (sc.mass_low + sc.mass_wall);
    P.cBH = sc.mass_wall / (sc.mass_high + sc.mass_wall);
    P.hx = (cfg->r_low + cfg->r_high) / 2.0f;
    P.relax_dt = cfg->dt / cfg->relax_dt_div;
    for (int k = 0; k < 4; ++k) P.roi[k] = cfg->roi[k];
    P.roi_vdt[0] = cfg->roi_velocity[0] * cfg->dt;  // FP32 products
    P.roi_vdt[1] = cfg->roi_velocity[1] * cfg->dt;
    P.relax_iters = cfg->relax_iters;
    P.q1 = (cfg->flags & TSS_FLAG_Q1_COMPAT) ? 1 : 0;
    P.merge = (cfg->flags & TSS_FLAG_MERGE) ? 1 : 0;
    P.tether_guard = (cfg->flags & TSS_FLAG_TETHER_GUARD) ? 1 : 0;
    P.older_place = (cfg->flags & TSS_FLAG_OLDER_PLACEMENT) ? 1 : 0;
    P.step0 = 0;
    P.Tle_r = sq_cutoff(P.r, true);
    P.Tlt_r = sq_cutoff(P.r, false);
    P.Tle_rh = sq_cutoff(P.rh, true);
    P.Tlt_rh = sq_cutoff(P.rh, false);
    recip_split(P.r, P.inv_hi.x, P.inv_lo.x);
    recip_split(P.rh, P.inv_hi.y, P.inv_lo.y);
    P.nLs = sc.n_low;
    P.CHs = cfg->dims_high[0] * cfg->dims_high[1];
    // FastArith's constants, from the same double values as the coefficients above
    P.fTor = make_float2(static_cast<float>(2.0 / r), static_cast<float>(2.0 / rh));
    P.fC = make_float2(static_cast<float>(10.0 / (14.0 * kPi * r * r)), static_cast<float>(10.0 / (14.0 * kPi * rh * rh)));
    P.fG = make_float2(static_cast<float>(-60.0 / (14.0 * kPi * r * r * r)),
                       static_cast<float>(-60.0 / (14.0 * kPi * rh * rh * rh)));
    const double hs[3] = {r, 0.5 * (r + rh), rh};
    float eps[3], kv[3];
    for (int k = 0; k < 3; ++k) {
        eps[k] = static_cast<float>(0.01 * hs[k] * hs[k]);
        kv[k] = static_cast<float>(2.0 * hs[k] * cfg->alpha * static_cast<double>(cfg->speed_sound));
    }
    P.fEps = make_float3(eps[0], eps[1], eps[2]);
    P.fKv = make_float3(kv[0], kv[1], kv[2]);
    P.fKw = static_cast<float>(0.02 * static_cast<double>(cfg->speed_sound) * cfg->speed_sound);
    return P;
}

void scene_runs(const SceneIn& sc, tss_footprint* f) {
    f->low_slots = sc.n_low;
    f->high_particles = 4LL * sc.n_low;
    f->low_cells = static_cast<int64_t>(sc.cfg->dims_low[0]) * sc.cfg->dims_low[1] + 1;
    f->high_cells = static_cast<int64_t>(sc.cfg->dims_high[0]) * sc.cfg->dims_high[1];
    f->wall_particles = sc.n_wall;
}

}  // namespace tss

extern "C" {

const char* tss_status_string(tss_status st) {
    switch (st) {
        case TSS_OK: return "ok";
        case TSS_INVALID_ARG: return "invalid argument";
        case TSS_OOM: return "out of memory";
        case TSS_CUDA_ERROR: return "CUDA error";
        case TSS_CAPACITY: return "particle pool capacity exceeded";
        case TSS_NUMERIC: return "NaN or Inf in the particle state";
        case TSS_GRID_INDEX: return "grid index check failed (inconsistent cell offsets)";
        case TSS_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

tss_status tss_config_init(tss_config* cfg, float xs, float ys, float xe, float ye, float effective_radius,
                           float effective_radius_high, float rest_density, float tait_coeff, float speed_sound,
                           float alpha, float tension_coefficient, float time_step) {
    if (!cfg) return TSS_INVALID_ARG;
    if (xs >= xe || ys >= ye) return TSS_INVALID_ARG;  // WCSPHConfig ctor, 2312-2316
    if (!(effective_radius > 0.0f) || !(effective_radius_high > 0.0f)) return TSS_INVALID_ARG;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->domain_origin[0] = xs;
    cfg->domain_origin[1] = ys;
    cfg->domain_end[0] = xe;
    cfg->domain_end[1] = ye;
    cfg->dims_low[0] = static_cast<int>(std::ceil((xe - xs) / effective_radius));
    cfg->dims_low[1] = static_cast<int>(std::ceil((ye - ys) / effective_radius));
    cfg->dims_high[0] = static_cast<int>(std::ceil((xe - xs) / effective_radius_high));
    cfg->dims_high[1] = static_cast<int>(std::ceil((ye - ys) / effective_radius_high));
    cfg->r_low = effective_radius;
    cfg->r_high = effective_radius_high;
    cfg->rest_density = rest_density;
    cfg->tait_b = tait_coeff;
    cfg->speed_sound = speed_sound;
    cfg->alpha = alpha;
    cfg->tension = tension_coefficient;
    cfg->dt = time_step;
    cfg->gravity = 9.81f;
    cfg->roi[0] = 0.5f;
    cfg->roi[1] = -INFINITY;
    cfg->roi[2] = INFINITY;
    cfg->roi[3] = INFINITY;
    cfg->relax_iters = 0;
    cfg->relax_dt_div = 10.0f;
    cfg->flags = TSS_FLAG_Q1_COMPAT;
    return TSS_OK;
}

}  // extern "C"

namespace {

// A single scene (tss_solver_create); pools and batches are created in pool.cu.
tss_status create_solver(const SceneIn& sc, int cap_high, tss_solver** out) {
    if (!out) return TSS_INVALID_ARG;
    *out = nullptr;
    if (!valid_cfg(sc.cfg) || sc.n_low < 0 || sc.n_wall < 0 || cap_high < 0) return TSS_INVALID_ARG;
    if ((sc.n_low > 0 && !sc.low_pos) || (sc.n_wall > 0 && !sc.wall_pos)) return TSS_INVALID_ARG;
    if (4LL * sc.n_low >= (1LL << 31) - 1) return TSS_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TSS_NO_DEVICE;

    tss_solver* s = new (std::nothrow) tss_solver();
    if (!s) return TSS_OOM;
    const int n_low = sc.n_low, n_wall = sc.n_wall;
    s->cfg = *sc.cfg;
    s->nL = n_low;
    s->capH = cap_high;
    s->slotsL = n_low;
    s->slotsH = 4 * n_low;
    s->nW = n_wall;
    s->CL = sc.cfg->dims_low[0] * sc.cfg->dims_low[1];
    s->CH = sc.cfg->dims_high[0] * sc.cfg->dims_high[1];
    s->carry = sc.cfg->relax_iters > 0;
    s->P = make_params(sc);
    s->P.slotsL = s->slotsL;
    s->P.slotsH = s->slotsH;
    s->P.capH = cap_high;

    // ---- one arena for everything ----
    Arena A;
    auto scale = [&](ScaleBufs& b, int cap, int slots) {
        A.add(&b.pos, cap);
        A.add(&b.vel, cap);
        A.add(&b.acc, cap);
        A.add(&b.npos, cap);
        A.add(&b.nvel, cap);
        A.add(&b.st, cap);
        A.add(&b.nst, cap);
        A.add(&b.id, cap);
        A.add(&b.nid, cap);
        A.add(&b.map, slots);
        A.add(&b.dens, cap);
        A.add(&b.pres, cap);
        A.add(&b.q, cap);
        A.add(&b.tr, cap);
        A.add(&b.nbr, static_cast<size_t>(kMaxNbr) * (cap > 0 ? cap : 1));
        A.add(&b.nnbr, cap);
        b.cap = cap > 0 ? cap : 1;
        A.add(&b.ndens, s->carry ? cap : 1);
        A.add(&b.npres, s->carry ? cap : 1);
    };
    scale(s->L, n_low, s->slotsL);
    scale(s->H, cap_high, s->slotsH);
    A.add(&s->L.cflag, s->CL);
    A.add(&s->H.cflag, 1);
    A.add(&s->wnear, s->CL);
    char* gL = nullptr;
    char* gH = nullptr;
    char* gW = nullptr;
    A.add(&gL, grid_bufs_bytes(n_low > 0 ? n_low : 1, s->CL));
    A.add(&gH, grid_bufs_bytes(cap_high > 0 ? cap_high : 1, s->CH));
    A.add(&gW, grid_bufs_bytes(n_wall > 0 ? n_wall : 1, s->CL));
    float2* wraw = nullptr;
    int32_t* wid = nullptr;
    A.add(&s->wpos, n_wall);
    A.add(&wraw, n_wall);
    A.add(&wid, n_wall);
    A.add(&s->cnt, 1);
    int* nW_dev = nullptr;
    A.add(&nW_dev, 4);
    A.add(&s->split_flag, n_low);
    A.add(&s->split_ids, n_low);
    s->split_ntiles = n_low > 0 ? (n_low + kSplitTile - 1) / kSplitTile : 1;
    A.add(&s->split_tile, s->split_ntiles);
    A.add(&s->relax_pos, s->carry ? cap_high : 1);
    A.add(&s->relax_vel, s->carry ? cap_high : 1);
    cudaError_t e = cudaMalloc(&s->arena, A.total());
    if (e != cudaSuccess) {
        tss_status st = e == cudaErrorMemoryAllocation ? TSS_OOM : TSS_CUDA_ERROR;
        delete s;
        return st;
    }
    s->arena_bytes = A.total();
    A.carve(s->arena);
    s->L.g = grid_bufs_carve(gL, n_low > 0 ? n_low : 1, s->CL);
    s->H.g = grid_bufs_carve(gH, cap_high > 0 ? cap_high : 1, s->CH);
    GridBufs gw = grid_bufs_carve(gW, n_wall > 0 ? n_wall : 1, s->CL);
    s->woff = gw.off;
    // the low-res gathers take one block per 256 particles (their count is fixed):
    // every block does one tile of work, which balances better than a capped
    // grid-stride launch
    s->blocksL = n_low > 0 ? (n_low + 255) / 256 : 1;
    s->blocksH = particle_blocks(cap_high > 0 ? cap_high : 1, 256);
    s->low_full = true;
    if (s->apply_launch(default_launch()) != TSS_OK) {
        delete s;
        return TSS_CUDA_ERROR;
    }

    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete s;
        return TSS_CUDA_ERROR;
    }
    cudaStream_t st = s->stream;
    // zero the whole arena: counts, maps (set to -1 below), pools
    e = cudaMemsetAsync(s->arena, 0, A.total(), st);
    if (e == cudaSuccess) launch_fill_i32(s->L.map, s->slotsL, -1, st);
    if (e == cudaSuccess) launch_fill_i32(s->H.map, s->slotsH, -1, st);
    if (e == cudaSuccess && n_low > 0) {
        e = cudaMemcpyAsync(s->L.npos, sc.low_pos, sizeof(float2) * n_low, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            if (sc.low_vel) e = cudaMemcpyAsync(s->L.nvel, sc.low_vel, sizeof(float2) * n_low, cudaMemcpyHostToDevice, st);
        }
        launch_iota(s->L.nid, n_low, st);
    }
    launch_set_counts(s->cnt, n_low, 0, st);
    // boundary grid, once (initBoundaries, 3205-3238): iota ids, low grid
    if (e == cudaSuccess && n_wall > 0) {
        e = cudaMemcpyAsync(wraw, sc.wall_pos, sizeof(float2) * n_wall, cudaMemcpyHostToDevice, st);
        launch_iota(wid, n_wall, st);
        k_set_int<<<1, 1, 0, st>>>(nW_dev, n_wall);
        ReorderArgs a{};
        a.src_pos = wraw;
        a.dst_pos = s->wpos;
        if (e == cudaSuccess)
            e = grid_build_enqueue(wraw, wid, nW_dev, n_wall, s->P.ox, s->P.oy, s->P.r, s->P.dimL[0], s->P.dimL[1],
                                   gw, a, &s->cnt->err, st);
        if (e == cudaSuccess) launch_wall_near(s->woff, s->wnear, s->P.dimL[0], s->P.dimL[1], st);
    }
    if (e == cudaSuccess) e = s->prime_keys(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        tss_status ret = e == cudaErrorMemoryAllocation ? TSS_OOM : TSS_CUDA_ERROR;
        delete s;
        return ret;
    }
    *out = s;
    return TSS_OK;
}

}  // namespace

extern "C" {

tss_status tss_solver_create(const tss_config* cfg, int n_low, const float* low_pos, const float* low_vel,
                             float mass_low, int cap_high, float mass_high, int n_wall, const float* wall_pos,
                             float mass_wall, tss_solver** out) {
    if (!out || !cfg) return TSS_INVALID_ARG;
    const SceneIn sc{cfg, n_low, low_pos, low_vel, mass_low, mass_high, n_wall, wall_pos, mass_wall};
    return create_solver(sc, cap_high, out);
}

void tss_solver_destroy(tss_solver* s) { delete s; }

tss_status tss_solver_step(tss_solver* s, int n_steps, void* stream) {
    if (!s || n_steps < 0) return TSS_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the default stream
    cudaError_t e;
    if ((e = s->enter(st)) != cudaSuccess) return s->cuda_fail(e, "order step");
    while (n_steps > 0) {
        int b = 0;  // bucket: 1 << b steps
        if (!s->profile) b = n_steps >= 8 ? 3 : (n_steps >= 4 ? 2 : (n_steps >= 2 ? 1 : 0));
        if (!s->exec[b]) {
            if ((e = s->ensure_side()) != cudaSuccess) return s->cuda_fail(e, "side stream");
            cudaStream_t cap = s->stream;
            if ((e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                return s->cuda_fail(e, "begin capture");
            cudaError_t e1 = cudaSuccess;
            for (int k = 0; k < (1 << b) && e1 == cudaSuccess; ++k) e1 = s->enqueue_step(cap);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(cap, &g);
            if (e1 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return s->cuda_fail(e1, "enqueue step");
            }
            if (e != cudaSuccess) return s->cuda_fail(e, "end capture");
            s->graph[b] = g;
            if ((e = cudaGraphInstantiate(&s->exec[b], g, 0)) != cudaSuccess) {
                s->drop_graph();
                return s->cuda_fail(e, "instantiate");
            }
        }
        if ((e = cudaGraphLaunch(s->exec[b], st)) != cudaSuccess) return s->cuda_fail(e, "graph launch");
        s->steps_issued += 1 << b;
        s->phys_low = s->live_low;  // the step's grid build dropped the retired scenes' entries
        n_steps -= 1 << b;
    }
    s->uploaded[0] = s->uploaded[1] = false;
    if ((e = s->leave(st)) != cudaSuccess) return s->cuda_fail(e, "record step");
    return TSS_OK;
}

tss_status tss_solver_sync(tss_solver* s) {
    if (!s) return TSS_INVALID_ARG;
    cudaError_t e = s->wait_idle();
    if (e != cudaSuccess) return s->cuda_fail(e, "synchronize");
    Counters c;
    if ((e = s->d2h(&c, s->cnt, sizeof(c))) != cudaSuccess)
        return s->cuda_fail(e, "read counters");
    if (c.err & kErrGridIndex) return s->fail(TSS_GRID_INDEX, "inconsistent grid offsets (an index check failed)");
    if (c.err & kErrCapacity) return s->fail(TSS_CAPACITY, "high-res pool capacity exceeded by a split");
    if (c.err & kErrNumeric) return s->fail(TSS_NUMERIC, "NaN/Inf density, pressure or acceleration");
    return TSS_OK;
}

tss_status tss_solver_counts(tss_solver* s, tss_counts* out) {
    if (!s || !out) return TSS_INVALID_ARG;
    cudaError_t e = s->wait_idle();
    Counters c;
    if (e == cudaSuccess) e = s->d2h(&c, s->cnt, sizeof(c));
    if (e != cudaSuccess) return s->cuda_fail(e, "counts");
    out->n_low = c.cur[0];
    out->n_high = c.cur[1] - c.dropped;  // removed entries wait in the list for the next build
    out->n_transient_low = out->n_high / 4;
    out->n_split_last = c.n_split;
    out->steps = c.steps;
    out->error_bits = c.err;
    out->n_removed_last = c.dropped;
    out->total_split = c.total_split;
    out->total_removed = c.total_removed;
    return TSS_OK;
}

namespace {

// Copy the first np list entries of a scale into the given host arrays (any may be null).
cudaError_t copy_list(tss_solver* s, int scale, int np, const tss_scale_state& o) {
    ScaleBufs& b = scale == 0 ? s->L : s->H;
    cudaError_t e = cudaSuccess;
    if (np == 0) return e;
    if (o.id) e = s->d2h(o.id, b.nid, sizeof(int32_t) * np);
    if (e == cudaSuccess && o.pos) e = s->d2h(o.pos, b.npos, sizeof(float2) * np);
    if (e == cudaSuccess && o.vel) e = s->d2h(o.vel, b.nvel, sizeof(float2) * np);
    if (e == cudaSuccess && o.state) e = s->d2h(o.state, b.nst, np);
    if (e == cudaSuccess && (o.dens || o.pres)) {
        if (s->carry) {
            if (o.dens) e = s->d2h(o.dens, b.ndens, sizeof(float) * np);
            if (e == cudaSuccess && o.pres) e = s->d2h(o.pres, b.npres, sizeof(float) * np);
        } else {
            // list order = last step's sorted order for the particles that existed then
            Counters cc;
            e = s->d2h(&cc, s->cnt, sizeof(cc));
            int m = (cc.steps > 0 && !s->uploaded[scale]) ? cc.sorted[scale] : 0;
            if (m > np) m = np;
            if (o.dens) {
                std::memset(o.dens, 0, sizeof(float) * np);
                if (e == cudaSuccess && m) e = s->d2h(o.dens, b.dens, sizeof(float) * m);
            }
            if (o.pres) {
                std::memset(o.pres, 0, sizeof(float) * np);
                if (e == cudaSuccess && m) e = s->d2h(o.pres, b.pres, sizeof(float) * m);
            }
        }
    }
    return e;
}

}  // namespace

// The list of a scale; entries removed in the last step (state 2, still in the
// list until the next grid build) are left out.
tss_status tss_solver_download(tss_solver* s, int scale, tss_scale_state* out) {
    if (!s || !out || (scale != 0 && scale != 1)) return TSS_INVALID_ARG;
    tss_counts c;
    tss_status st = tss_solver_counts(s, &c);
    if (st != TSS_OK) return st;
    const int n = scale == 0 ? c.n_low : c.n_high;
    const int removed = scale == 1 ? c.n_removed_last : 0;
    if (out->n < n) {
        out->n = n;
        return s->fail(TSS_INVALID_ARG, "download buffer too small");
    }
    out->n = n;
    cudaError_t e;
    if (removed == 0) {
        e = copy_list(s, scale, n, *out);
    } else {
        const size_t np = static_cast<size_t>(n) + removed;
        std::vector<int32_t> id(np);
        std::vector<float> pos(2 * np), vel(2 * np), dens(np), pres(np);
        std::vector<uint8_t> stt(np);
        tss_scale_state t{static_cast<int>(np), id.data(), pos.data(), vel.data(), stt.data(), dens.data(), pres.data()};
        e = copy_list(s, scale, static_cast<int>(np), t);
        int m = 0;
        for (size_t i = 0; i < np && e == cudaSuccess; ++i) {
            if (stt[i] == 2) continue;
            if (m >= n) break;
            if (out->id) out->id[m] = id[i];
            if (out->pos) {
                out->pos[2 * m] = pos[2 * i];
                out->pos[2 * m + 1] = pos[2 * i + 1];
            }
            if (out->vel) {
                out->vel[2 * m] = vel[2 * i];
                out->vel[2 * m + 1] = vel[2 * i + 1];
            }
            if (out->state) out->state[m] = stt[i];
            if (out->dens) out->dens[m] = dens[i];
            if (out->pres) out->pres[m] = pres[i];
            ++m;
        }
    }
    if (e != cudaSuccess) return s->cuda_fail(e, "download");
    return TSS_OK;
}

tss_status tss_solver_upload(tss_solver* s, int scale, const tss_scale_state* in) {
    if (!s || !in || (scale != 0 && scale != 1)) return TSS_INVALID_ARG;
    const int n = in->n;
    const int cap = scale == 0 ? s->nL : s->capH;
    const int slots = scale == 0 ? s->slotsL : s->slotsH;
    if (n < 0 || n > cap) return s->fail(TSS_INVALID_ARG, "count exceeds capacity");
    const int64_t want_low = s->batched ? s->live_low : s->nL;
    if (scale == 0 && n != want_low) return s->fail(TSS_INVALID_ARG, "the low-res count is fixed by the scenes");
    if (n > 0 && (!in->id || !in->pos || !in->state)) return s->fail(TSS_INVALID_ARG, "missing arrays");
    std::vector<char> seen(static_cast<size_t>(slots), 0);
    for (int i = 0; i < n; ++i) {
        const int id = in->id[i];
        if (id < 0 || id >= slots || seen[id]) return s->fail(TSS_INVALID_ARG, "ids must be unique and in range");
        if (s->batched) {  // the slot must belong to an admitted scene
            const int low = scale == 0 ? id : id >> 2;
            const int sc = s->h_page_scene[static_cast<size_t>(low) >> 8];
            const SceneRec& r = s->scenes[sc];
            if (!r.live || low < r.sb || low >= r.sb + r.n_low)
                return s->fail(TSS_INVALID_ARG, "id outside the admitted scenes");
        }
        seen[id] = 1;
    }
    cudaError_t e = s->wait_idle();
    ScaleBufs& b = scale == 0 ? s->L : s->H;
    if (e == cudaSuccess && n > 0) {
        e = s->h2d(b.nid, in->id, sizeof(int32_t) * n);
        if (e == cudaSuccess) e = s->h2d(b.npos, in->pos, sizeof(float2) * n);
        if (e == cudaSuccess) {
            if (in->vel) e = s->h2d(b.nvel, in->vel, sizeof(float2) * n);
            else e = s->memset0(b.nvel, sizeof(float2) * n);
        }
        if (e == cudaSuccess) e = s->h2d(b.nst, in->state, n);
        if (e == cudaSuccess && s->carry) {
            if (in->dens) e = s->h2d(b.ndens, in->dens, sizeof(float) * n);
            else e = s->memset0(b.ndens, sizeof(float) * n);
            if (e == cudaSuccess) {
                if (in->pres) e = s->h2d(b.npres, in->pres, sizeof(float) * n);
                else e = s->memset0(b.npres, sizeof(float) * n);
            }
        }
    }
    if (e == cudaSuccess && slots > 0) {
        launch_fill_i32(b.map, slots, -1, s->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        Counters c;
        e = s->d2h(&c, s->cnt, sizeof(c));
        if (e == cudaSuccess) {
            int nL = scale == 0 ? n : c.cur[0];
            int nH = scale == 1 ? n : c.cur[1];
            launch_set_counts(s->cnt, nL, nH, s->stream);
            if (scale == 0) s->phys_low = n;
            e = s->prime_keys(s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        }
    }
    if (e != cudaSuccess) return s->cuda_fail(e, "upload");
    s->uploaded[scale] = true;
    return TSS_OK;
}

tss_status tss_solver_get_fresh(tss_solver* s, int* n, int32_t* parents) {
    if (!s || !n) return TSS_INVALID_ARG;
    Counters c;
    cudaError_t e = s->wait_idle();
    if (e == cudaSuccess) e = s->d2h(&c, s->cnt, sizeof(c));
    if (e == cudaSuccess && parents && c.n_fresh > 0)
        e = s->d2h(parents, s->split_ids, sizeof(int32_t) * c.n_fresh);
    if (e != cudaSuccess) return s->cuda_fail(e, "get fresh");
    *n = c.n_fresh;
    return TSS_OK;
}

tss_status tss_solver_set_fresh(tss_solver* s, int n, const int32_t* parents) {
    if (!s || n < 0 || n > s->nL || (n > 0 && !parents)) return TSS_INVALID_ARG;
    for (int i = 0; i < n; ++i)
        if (parents[i] < 0 || parents[i] >= s->slotsL) return s->fail(TSS_INVALID_ARG, "parent id out of range");
    cudaError_t e = s->wait_idle();
    if (e == cudaSuccess && n > 0) e = s->h2d(s->split_ids, parents, sizeof(int32_t) * n);
    if (e == cudaSuccess) {
        k_set_fresh<<<1, 1, 0, s->stream>>>(s->cnt, n);
        e = cudaStreamSynchronize(s->stream);
    }
    if (e != cudaSuccess) return s->cuda_fail(e, "set fresh");
    return TSS_OK;
}

tss_status tss_solver_copy(tss_solver* s, int scale, int which, void* dst, size_t count, size_t* written) {
    if (!s || (scale != 0 && scale != 1)) return TSS_INVALID_ARG;
    Counters c;
    cudaError_t e = s->wait_idle();
    if (e == cudaSuccess) e = s->d2h(&c, s->cnt, sizeof(c));
    if (e != cudaSuccess) return s->cuda_fail(e, "copy");
    ScaleBufs& b = scale == 0 ? s->L : s->H;
    // particles sorted in the last step: the count before its splits
    const int n_sorted = c.steps > 0 ? c.sorted[scale] : 0;
    const void* src = nullptr;
    size_t n = 0, esz = 4;
    switch (which) {
        case TSS_BUF_SORTED_ID: src = b.id; n = n_sorted; break;
        case TSS_BUF_CELL_OFFSET: src = b.g.off; n = static_cast<size_t>(b.g.ncells) + 1; break;
        case TSS_BUF_DENSITY: src = b.dens; n = n_sorted; break;
        case TSS_BUF_PRESSURE: src = b.pres; n = n_sorted; break;
        case TSS_BUF_ACCEL: src = b.acc; n = 2 * static_cast<size_t>(n_sorted); break;
        case TSS_BUF_SPLIT:
            if (scale != 0) return TSS_INVALID_ARG;
            src = s->split_ids;
            n = c.n_split;
            break;
        case TSS_BUF_WALL_CELL_OFFSET:
            if (scale != 0) return TSS_INVALID_ARG;
            src = s->woff;
            n = static_cast<size_t>(s->CL) + 1;
            break;
        default: return TSS_INVALID_ARG;
    }
    if (written) *written = n;
    if (!dst) return TSS_OK;
    if (count < n) return s->fail(TSS_INVALID_ARG, "destination too small");
    if (n && (e = s->d2h(dst, src, n * esz)) != cudaSuccess) return s->cuda_fail(e, "copy");
    return TSS_OK;
}

tss_status tss_solver_device_buffers(tss_solver* s, tss_buffers* out) {
    if (!s || !out) return TSS_INVALID_ARG;
    const ScaleBufs* b[2] = {&s->L, &s->H};
    for (int k = 0; k < 2; ++k) {
        out->pos[k] = reinterpret_cast<const float*>(b[k]->npos);
        out->vel[k] = reinterpret_cast<const float*>(b[k]->nvel);
        out->dens[k] = b[k]->dens;
        out->id[k] = b[k]->nid;
        out->state[k] = b[k]->nst;
    }
    out->counts = reinterpret_cast<const int*>(reinterpret_cast<const char*>(s->cnt) + offsetof(Counters, cur));
    return TSS_OK;
}

tss_status tss_solver_profile(tss_solver* s, int enable) {
    if (!s) return TSS_INVALID_ARG;
    const bool want = enable != 0;
    if (want == s->profile) return TSS_OK;
    cudaError_t e = s->wait_idle();
    if (e != cudaSuccess) return s->cuda_fail(e, "profile");
    if (want)
        for (auto& x : s->ev)
            if (!x && (e = cudaEventCreate(&x)) != cudaSuccess) return s->cuda_fail(e, "event create");
    s->profile = want;
    s->drop_graph();  // re-captured with (or without) the event nodes at the next step
    return TSS_OK;
}

tss_status tss_solver_stage_times(tss_solver* s, float* ms, int n) {
    if (!s || !ms || n < TSS_NUM_STAGES) return TSS_INVALID_ARG;
    if (!s->profile) return s->fail(TSS_INVALID_ARG, "profiling is off");
    cudaError_t e = s->wait_idle();
    for (int k = 0; k < TSS_NUM_STAGES && e == cudaSuccess; ++k) e = cudaEventElapsedTime(&ms[k], s->ev[k], s->ev[k + 1]);
    if (e != cudaSuccess) return s->cuda_fail(e, "stage times");
    return TSS_OK;
}

// The device-side addresses of a read-back's page-locked host buffers (an error for
// memory the GPU cannot reach, which is refused before any kernel touches it).
static tss_status read_targets(tss_solver* s, float* host_low, int cap_low, float* host_high, int cap_high,
                               int* counts, void* dev[3]) {
    if (!counts || cap_low < 0 || cap_high < 0 || (cap_low > 0 && !host_low) || (cap_high > 0 && !host_high))
        return TSS_INVALID_ARG;
    void* host[3] = {host_low, host_high, counts};
    for (int k = 0; k < 3; ++k) {
        dev[k] = nullptr;
        if (!host[k]) continue;
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, host[k]) != cudaSuccess || a.type != cudaMemoryTypeHost ||
            cudaHostGetDevicePointer(&dev[k], host[k], 0) != cudaSuccess || !dev[k]) {
            cudaGetLastError();  // clear the failed query
            return s->fail(TSS_INVALID_ARG, "read_positions: host buffers must be page-locked and mapped");
        }
    }
    return TSS_OK;
}

static int read_blocks(int n) { return std::max(1, std::min(particle_blocks(std::max(n, 1), 256), 4 * sm_count())); }

tss_status tss_solver_read_positions(tss_solver* s, float* host_low, int cap_low, float* host_high, int cap_high,
                                     int* counts, void* stream) {
    if (!s) return TSS_INVALID_ARG;
    void* dev[3];
    const tss_status st = read_targets(s, host_low, cap_low, host_high, cap_high, counts, dev);
    if (st != TSS_OK) return st;
    const cudaStream_t cs = static_cast<cudaStream_t>(stream);
    cudaError_t e = s->enter(cs);
    if (e == cudaSuccess) {
        k_read_positions<<<read_blocks(std::max(cap_low, cap_high)), 256, 0, cs>>>(
            s->L.npos, s->H.npos, &s->cnt->cur[0], static_cast<float2*>(dev[0]), cap_low,
            static_cast<float2*>(dev[1]), cap_high, static_cast<int*>(dev[2]));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = s->leave(cs);
    return e == cudaSuccess ? TSS_OK : s->cuda_fail(e, "read_positions");
}

tss_status tss_solver_read_positions_async(tss_solver* s, float* host_low, int cap_low, float* host_high,
                                           int cap_high, int* counts, void* stream, int64_t* ticket) {
    if (!s || !ticket) return TSS_INVALID_ARG;
    void* dev[3];
    tss_status st = read_targets(s, host_low, cap_low, host_high, cap_high, counts, dev);
    if (st != TSS_OK) return st;
    auto& rb = s->rb;
    cudaError_t e = cudaSuccess;
    if (!rb.stream) {  // first call: events and the stream
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
            e = cudaEventCreateWithFlags(&rb.staged[b], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&rb.done[b], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&rb.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return s->cuda_fail(e, "read_positions_async");
    }
    // staging buffers for what the caller reads (a pool's lists can be far longer);
    // grown when a call asks for more, once the copies in flight are done
    cap_low = std::min(cap_low, s->nL);
    cap_high = std::min(cap_high, s->capH);
    if (!rb.mem || cap_low > rb.cap_low || cap_high > rb.cap_high) {
        if (rb.mem) {
            if ((e = cudaStreamSynchronize(rb.stream)) != cudaSuccess) return s->cuda_fail(e, "read_positions_async");
            cudaFree(rb.mem);
            rb.mem = nullptr;
        }
        rb.cap_low = std::max(rb.cap_low, cap_low);
        rb.cap_high = std::max(rb.cap_high, cap_high);
        const size_t per = sizeof(float2) * (static_cast<size_t>(rb.cap_low) + rb.cap_high) + 16;
        if ((e = cudaMalloc(&rb.mem, 2 * per)) != cudaSuccess) {
            rb.cap_low = rb.cap_high = 0;
            return s->cuda_fail(e, "read_positions_async");
        }
        for (int b = 0; b < 2; ++b) {
            char* base = static_cast<char*>(rb.mem) + b * per;
            rb.counts[b] = reinterpret_cast<int*>(base);
            rb.low[b] = reinterpret_cast<float2*>(base + 16);
            rb.high[b] = rb.low[b] + rb.cap_low;
        }
    }
    const int b = static_cast<int>(rb.issued & 1);
    const cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // the buffer's previous host copy (two calls ago) must be done before it is refilled
    e = s->enter(cs);
    if (e == cudaSuccess && rb.issued >= 2) e = cudaStreamWaitEvent(cs, rb.done[b], 0);
    if (e == cudaSuccess) {
        k_read_positions<<<read_blocks(std::max(cap_low, cap_high)), 256, 0, cs>>>(
            s->L.npos, s->H.npos, &s->cnt->cur[0], rb.low[b], cap_low, rb.high[b], cap_high, rb.counts[b]);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(rb.staged[b], cs);
    if (e == cudaSuccess) e = s->leave(cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(rb.stream, rb.staged[b], 0);
    // A single scene's lists go by copy engine, leaving the SMs to the next step:
    // the low-res list (it always holds all nL particles), the high-res list at the
    // caller's capacity (its length is on the device; entries past it are stale),
    // then the two lengths.  On the developed 1M dam break (1M + 1M particles) that
    // took the end-to-end rate from 3.74 to 4.02 G particle-steps/s against moving
    // the high-res list by a kernel, which shared the SMs with the next step.  A
    // batch's lists (their lengths on the device) go by a kernel.
    int kernel_low = cap_low;
    if (e == cudaSuccess && !s->batched && cap_low > 0) {
        e = cudaMemcpyAsync(host_low, rb.low[b], sizeof(float2) * static_cast<size_t>(cap_low),
                            cudaMemcpyDeviceToHost, rb.stream);
        kernel_low = 0;
    }
    if (e == cudaSuccess && !s->batched) {
        if (cap_high > 0)
            e = cudaMemcpyAsync(host_high, rb.high[b], sizeof(float2) * static_cast<size_t>(cap_high),
                                cudaMemcpyDeviceToHost, rb.stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(counts, rb.counts[b], 2 * sizeof(int), cudaMemcpyDeviceToHost, rb.stream);
    } else if (e == cudaSuccess) {
        k_read_positions<<<read_blocks(std::max(kernel_low, cap_high)), 256, 0, rb.stream>>>(
            rb.low[b], rb.high[b], rb.counts[b], static_cast<float2*>(dev[0]), kernel_low,
            static_cast<float2*>(dev[1]), cap_high, static_cast<int*>(dev[2]));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(rb.done[b], rb.stream);
    if (e != cudaSuccess) return s->cuda_fail(e, "read_positions_async");
    *ticket = rb.issued++;
    return TSS_OK;
}

tss_status tss_solver_read_wait(tss_solver* s, int64_t ticket) {
    if (!s || ticket < 0 || ticket >= s->rb.issued) return TSS_INVALID_ARG;
    // buffer ticket & 1 was last used by ticket or a later read-back on the same
    // in-order stream: its completion implies this one's
    const cudaError_t e = cudaEventSynchronize(s->rb.done[ticket & 1]);
    return e == cudaSuccess ? TSS_OK : s->cuda_fail(e, "read_wait");
}

tss_status tss_solver_get_launch(tss_solver* s, tss_launch* out) {
    if (!s || !out) return TSS_INVALID_ARG;
    *out = s->launch;
    return TSS_OK;
}

tss_status tss_solver_set_launch(tss_solver* s, const tss_launch* in) {
    if (!s || !in) return TSS_INVALID_ARG;
    // steps run on callers' streams: wait for all of them before the old graphs go
    cudaError_t e = s->wait_idle();
    if (e != cudaSuccess) return s->cuda_fail(e, "set launch");
    return s->apply_launch(*in);
}

tss_status tss_solver_set_arith(tss_solver* s, int mode) {
    if (!s || (mode != TSS_ARITH_EXACT && mode != TSS_ARITH_FAST)) return TSS_INVALID_ARG;
    if (mode == s->arith) return TSS_OK;
    // the old graphs may still run on callers' streams
    cudaError_t e = s->wait_idle();
    if (e != cudaSuccess) return s->cuda_fail(e, "set arith");
    s->arith = mode;
    return s->apply_launch(s->launch);  // grids of persistent shapes follow the kernels' occupancy
}

tss_status tss_solver_get_arith(tss_solver* s, int* mode) {
    if (!s || !mode) return TSS_INVALID_ARG;
    *mode = s->arith;
    return TSS_OK;
}

// Stage of each gather in the profiled step (tss_solver_stage_times).
static const int kGatherStage[TSS_NUM_GATHERS] = {3, 4, 5, 7};

tss_status tss_solver_autotune(tss_solver* s, int steps_per_trial, tss_launch* best, int* steps_taken) {
    if (!s || !best || steps_per_trial < 1) return TSS_INVALID_ARG;
    const bool was_profiling = s->profile;
    const tss_launch before = s->launch;
    tss_status st = tss_solver_profile(s, 1);
    if (st != TSS_OK) return st;
    // The default shape is timed first and a candidate replaces the incumbent of a
    // gather only when it is faster by more than kMargin: trial steps are few and
    // early (a scale may still be nearly empty), and a shape that wins by noise
    // can lose once the lists fill.
    constexpr float kMargin = 0.05f;
    tss_launch b = default_launch();
    float best_ms[TSS_NUM_GATHERS];
    for (float& x : best_ms) x = 3.0e38f;
    int taken = 0;
    // candidates in order: the default (256 threads, covering, a particle per
    // thread) first; the last takes a particle per warp
    constexpr int kCand = 7;
    const int cand_threads[kCand] = {256, 128, 64, 256, 128, 64, 256};
    const int cand_pers[kCand] = {0, 0, 0, 1, 1, 1, 0};
    const int cand_warp[kCand] = {0, 0, 0, 0, 0, 0, 1};
    for (int ci = 0; ci < kCand && st == TSS_OK; ++ci) {
        tss_launch c{};
        for (int g = 0; g < TSS_NUM_GATHERS; ++g) {
            c.threads[g] = cand_threads[ci];
            c.persistent[g] = cand_pers[ci];
            c.per_warp[g] = cand_warp[ci];
        }
        if ((st = s->apply_launch(c)) != TSS_OK) break;
        // one untimed step captures the graph
        if ((st = tss_solver_step(s, 1, s->stream)) != TSS_OK) break;
        ++taken;
        float sum[TSS_NUM_GATHERS] = {};
        for (int k = 0; k < steps_per_trial && st == TSS_OK; ++k) {
            if ((st = tss_solver_step(s, 1, s->stream)) != TSS_OK) break;
            ++taken;
            float ms[TSS_NUM_STAGES];
            if ((st = tss_solver_stage_times(s, ms, TSS_NUM_STAGES)) != TSS_OK) break;
            for (int g = 0; g < TSS_NUM_GATHERS; ++g) sum[g] += ms[kGatherStage[g]];
        }
        if (st != TSS_OK) break;
        for (int g = 0; g < TSS_NUM_GATHERS; ++g)
            if (ci == 0 || sum[g] < (1.0f - kMargin) * best_ms[g]) {
                best_ms[g] = sum[g];
                b.threads[g] = c.threads[g];
                b.persistent[g] = c.persistent[g];
                b.per_warp[g] = c.per_warp[g];
            }
    }
    // The per-gather choice was timed stage by stage in the profiled (sequential)
    // step graph; an unprofiled step runs the grid builds and the densities as
    // parallel branches, where shapes overlap differently.  So the whole step is
    // timed unprofiled with the per-gather choice, the default shape and one
    // particle per warp throughout, and the fastest of the three is kept.
    if (st == TSS_OK) st = tss_solver_profile(s, 0);
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (st == TSS_OK && (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess))
        st = s->fail(TSS_CUDA_ERROR, "event create");
    tss_launch whole[3] = {b, default_launch(), default_launch()};
    for (int g = 0; g < TSS_NUM_GATHERS; ++g) whole[2].per_warp[g] = 1;
    float whole_best = 3.0e38f;
    tss_launch pick = b;
    for (int wi = 0; wi < 3 && st == TSS_OK; ++wi) {
        if ((st = s->apply_launch(whole[wi])) != TSS_OK) break;
        if ((st = tss_solver_step(s, 1, s->stream)) != TSS_OK) break;  // captures the graph
        ++taken;
        if (cudaEventRecord(t0, s->stream) != cudaSuccess) {
            st = s->fail(TSS_CUDA_ERROR, "event record");
            break;
        }
        for (int k = 0; k < steps_per_trial && st == TSS_OK; ++k) {
            st = tss_solver_step(s, 1, s->stream);
            ++taken;
        }
        if (st != TSS_OK) break;
        float ms = 0.0f;
        if (cudaEventRecord(t1, s->stream) != cudaSuccess || cudaEventSynchronize(t1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) {
            st = s->fail(TSS_CUDA_ERROR, "event timing");
            break;
        }
        if (wi == 0 || ms < (1.0f - kMargin) * whole_best) {
            whole_best = ms;
            pick = whole[wi];
        }
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    b = pick;
    if (st == TSS_OK) st = tss_solver_sync(s);  // a numeric or capacity error of the trial steps
    if (st != TSS_OK) {
        const std::string why = s->err;
        s->apply_launch(before);
        tss_solver_profile(s, was_profiling ? 1 : 0);
        s->err = why;
        return st;
    }
    if ((st = s->apply_launch(b)) != TSS_OK) return st;
    if ((st = tss_solver_profile(s, was_profiling ? 1 : 0)) != TSS_OK) return st;
    *best = b;
    if (steps_taken) *steps_taken = taken;
    return TSS_OK;
}

tss_status tss_solver_last_error(tss_solver* s, char* buf, int len) {
    if (!s || !buf || len <= 0) return TSS_INVALID_ARG;
    std::snprintf(buf, static_cast<size_t>(len), "%s", s->err.c_str());
    return TSS_OK;
}

}  // extern "C"
