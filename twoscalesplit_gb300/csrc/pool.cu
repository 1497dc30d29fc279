// pool.cu -- pools of scenes: one solver handle whose device arrays are sized for
// capacities and whose scenes are admitted and retired between steps, and the
// fixed batches built on them (tss_batch_create).
//
// No counterpart in the reference, which held one scene per process
// (TwoScale2D/WCSPHSolver.cu:2728, activeID in a function static).  Every scene
// keeps the reference's per-scene semantics: its particles only meet particles of
// its own grid, because each scene owns a contiguous run of cells of the global
// cell space and its grid windows are clamped to its own grid.
//
// Layout.  Each resource is one linear device array, handed out in pages by a
// first-fit allocator (extent.hpp):
//   low-res slots    a scene's particle i has slot sb + i; its children 4(sb+i)+c.
//                    page_scene[slot / TSS_POOL_SLOT_PAGE] names the owner, and the
//                    grid reorder writes each sorted particle's scene from it
//   low/high cells   the scene's grids at cbL / cbH; the low run has one cell more
//                    than the grid, so the scene's wall offset table [cbL, cbL + C]
//                    never shares its end entry with the next scene
//   walls            the scene's walls at wb, sorted by (cell, id) within the
//                    scene at admission, with scene-local offsets
// The particle lists are shared and compact: an admission appends the scene's
// particles (and their next-build keys) to the low-res list; a retirement sets the
// keys of its entries to -1 and takes them out of the cell counts, so the next
// grid build drops them and the list is compact again.
//
// Extraction.  After a step the lists hold, in order, the particles sorted in that
// step (grouped by scene, because each scene's cells are one run of the global
// order) and then the children created in it (grouped by scene too, because the
// split compaction follows the sorted low-res order).  A scene's state is therefore
// three contiguous runs, found from the cell offsets and a count of split flags.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "solver_impl.cuh"

using namespace tss;

namespace {

constexpr int kSlotPageShift = 8;
static_assert((1 << kSlotPageShift) == TSS_POOL_SLOT_PAGE, "slot page");

// Append a scene's low-res particles at list entries [base, base + n): ids, states,
// carried density/pressure, and the keys of the next grid build.  Positions and
// velocities were copied there already.
__global__ void k_admit_low(const float2* __restrict__ npos, int32_t* __restrict__ nid, uint8_t* __restrict__ nst,
                            float* ndens, float* npres, int base, int n, int sb, Params P, GridBufs g) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = base + i;
        nid[k] = sb + i;
        nst[k] = 0;
        if (ndens) {
            ndens[k] = 0.0f;
            npres[k] = 0.0f;
        }
        grid_key(g.count, g.key, g.rank, g.tile_sum, k, P.cbL + cell_hash(npos[k], P.ox, P.oy, P.r, P.dimL[0], P.dimL[1]));
    }
}

// Take the list entries of low-res slots [lo, hi) out of the next grid build.
__global__ void k_retire(const int32_t* __restrict__ nid, const int* __restrict__ n_ptr, int cap, int shift, int lo,
                         int hi, GridBufs g, int32_t* map, int slots) {
    const int n = min(*n_ptr, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int id = nid[i];
        const int low = id >> shift;
        if (low < lo || low >= hi) continue;
        const int c = g.key[i];
        if (c >= 0 && c < g.ncells) {
            atomicSub(&g.count[c], 1u);
            atomicSub(&g.tile_sum[static_cast<unsigned>(c) / kScanTile], 1u);
        }
        g.key[i] = -1;
        if (map && id >= 0 && id < slots) map[id] = -1;
    }
}

// Split flags of the last step before the scene's first sorted low-res entry
// (out[0]) and among its entries (out[1]).
__global__ void k_count_splits(const uint8_t* __restrict__ flag, const int* __restrict__ offL, int cb, int ncells,
                               const Counters* __restrict__ cnt, unsigned* out, int32_t* d_counts) {
    const int lf = offL[cb], le = min(offL[cb + ncells], cnt->sorted[0]);
    if (blockIdx.x == 0 && threadIdx.x == 0) d_counts[2] = 0;  // k_extract counts non-finite particles into it
    unsigned a = 0, b = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < le; i += gridDim.x * blockDim.x) {
        const unsigned f = flag[i] != 0;
        if (i < lf) a += f;
        else b += f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(&out[0], a);
        if (b) atomicAdd(&out[1], b);
    }
}

struct ExtractArgs {
    // the scene
    int sb, n_low, cbL, CLs, cbH, CHs;
    // list and sorted arrays
    const float2 *lpos, *lvel, *hpos, *hvel;
    const uint8_t *lst, *hst;
    const int32_t *lid, *hid;
    const float *ldens, *lpres, *hdens, *hpres;  // density/pressure per list entry (sorted arrays or carried)
    bool kid_dens;                               // carried arrays: children's entries are valid (zero)
    const int *offL, *offH;
    const Counters* cnt;
    const unsigned* splits;                      // k_count_splits output
    tss_scene_result dst;
    int32_t* d_counts;
};

__global__ void k_extract(ExtractArgs a) {
    const int lf = a.offL[a.cbL], le = a.offL[a.cbL + a.CLs];
    const int hf = a.offH[a.cbH], he = a.offH[a.cbH + a.CHs];
    const int nl = le - lf, ns = he - hf;
    const int nH_sorted = a.cnt->sorted[1], nH_list = a.cnt->cur[1];
    int kf = nH_sorted + 4 * static_cast<int>(a.splits[0]);
    int nk = 4 * static_cast<int>(a.splits[1]);
    if (kf > nH_list) kf = nH_list;
    if (kf + nk > nH_list) nk = nH_list - kf;
    const int64_t total = 5LL * a.n_low;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.d_counts[0] = nl;
        a.d_counts[1] = ns + nk;
    }
    for (int64_t tt = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; tt < total;
         tt += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (tt < a.n_low) {
            const int t = static_cast<int>(tt);
            const int k = lf + t;
            if (t >= nl || t >= a.dst.cap[0] || k < 0 || k >= a.cnt->sorted[0]) continue;
            if (a.dst.id[0]) a.dst.id[0][t] = a.lid[k] - a.sb;
            if (a.dst.pos[0]) reinterpret_cast<float2*>(a.dst.pos[0])[t] = a.lpos[k];
            if (a.dst.vel[0]) reinterpret_cast<float2*>(a.dst.vel[0])[t] = a.lvel[k];
            if (a.dst.state[0]) a.dst.state[0][t] = a.lst[k];
            if (a.dst.dens[0]) a.dst.dens[0][t] = a.ldens[k];
            if (a.dst.pres[0]) a.dst.pres[0][t] = a.lpres[k];
            const float2 p = a.lpos[k], v = a.lvel[k];
            if (!(isfinite(p.x) && isfinite(p.y) && isfinite(v.x) && isfinite(v.y) && isfinite(a.ldens[k])))
                atomicAdd(&a.d_counts[2], 1);
        } else {
            const int j = static_cast<int>(tt - a.n_low);
            if (j >= ns + nk || j >= a.dst.cap[1]) continue;
            const bool kid = j >= ns;
            const int k = kid ? kf + (j - ns) : hf + j;
            if (k < 0 || k >= (kid ? nH_list : nH_sorted)) continue;
            if (a.dst.id[1]) a.dst.id[1][j] = a.hid[k] - 4 * a.sb;
            if (a.dst.pos[1]) reinterpret_cast<float2*>(a.dst.pos[1])[j] = a.hpos[k];
            if (a.dst.vel[1]) reinterpret_cast<float2*>(a.dst.vel[1])[j] = a.hvel[k];
            if (a.dst.state[1]) a.dst.state[1][j] = a.hst[k];
            const bool dv = !kid || a.kid_dens;
            if (a.dst.dens[1]) a.dst.dens[1][j] = dv ? a.hdens[k] : 0.0f;
            if (a.dst.pres[1]) a.dst.pres[1][j] = dv ? a.hpres[k] : 0.0f;
            const float2 p = a.hpos[k], v = a.hvel[k];
            if (!(isfinite(p.x) && isfinite(p.y) && isfinite(v.x) && isfinite(v.y) && (!dv || isfinite(a.hdens[k]))))
                atomicAdd(&a.d_counts[2], 1);
        }
    }
}

bool pool_cfg_ok(const tss_pool_config& c) {
    return c.low_slots >= TSS_POOL_SLOT_PAGE && c.low_slots <= (1LL << 29) && c.high_particles >= 0 &&
           c.high_particles < (1LL << 31) - 1 && c.low_cells >= TSS_POOL_CELL_PAGE &&
           c.low_cells < (1LL << 31) - 2 && c.high_cells >= TSS_POOL_CELL_PAGE && c.high_cells < (1LL << 31) - 2 &&
           c.wall_particles >= 0 && c.wall_particles < (1LL << 31) - 1 && c.max_scenes >= 1 &&
           c.max_scenes <= TSS_POOL_MAX_SCENES && c.relax_iters >= 0 && c.relax_iters <= 64;
}

int64_t round_down(int64_t x, int64_t page) { return (x / page) * page; }

// Lay out a pool's arena on the handle (pointers relative to base; base == nullptr
// only sizes it).  Capacities are rounded down to whole pages.
struct PoolPlan {
    char *gL = nullptr, *gH = nullptr, *gW = nullptr;
};

void plan_pool(tss_solver* s, const tss_pool_config& c, Arena& A, PoolPlan& pp) {
    const int Ls = static_cast<int>(round_down(c.low_slots, TSS_POOL_SLOT_PAGE));
    const int Hc = static_cast<int>(c.high_particles);
    const int CLc = static_cast<int>(round_down(c.low_cells, TSS_POOL_CELL_PAGE));
    const int CHc = static_cast<int>(round_down(c.high_cells, TSS_POOL_CELL_PAGE));
    const int Wc = static_cast<int>(round_down(c.wall_particles, TSS_POOL_WALL_PAGE));
    s->batched = true;
    s->nL = Ls;
    s->capH = Hc;
    s->slotsL = Ls;
    s->slotsH = 4 * Ls;
    s->CL = CLc;
    s->CH = CHc;
    s->capW = Wc;
    s->nW = Wc;
    s->carry = c.relax_iters > 0;
    s->S = c.max_scenes;
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
    scale(s->L, Ls, s->slotsL);
    scale(s->H, Hc > 0 ? Hc : 1, s->slotsH);
    A.add(&s->L.cflag, CLc);
    A.add(&s->H.cflag, 1);
    A.add(&s->wnear, CLc);
    A.add(&pp.gL, grid_bufs_bytes(Ls, CLc));
    A.add(&pp.gH, grid_bufs_bytes(Hc > 0 ? Hc : 1, CHc));
    A.add(&pp.gW, grid_bufs_bytes(Wc > 0 ? Wc : 1, CLc));
    A.add(&s->wpos, Wc);
    A.add(&s->wraw, Wc);
    A.add(&s->wid, Wc);
    A.add(&s->cnt, 1);
    A.add(&s->split_flag, Ls);
    A.add(&s->split_ids, Ls);
    s->split_ntiles = (Ls + kSplitTile - 1) / kSplitTile;
    A.add(&s->split_tile, s->split_ntiles);
    A.add(&s->relax_pos, s->carry ? Hc : 1);
    A.add(&s->relax_vel, s->carry ? Hc : 1);
    A.add(&s->d_table, c.max_scenes);
    A.add(&s->scL, Ls);
    A.add(&s->scH, Hc > 0 ? Hc : 1);
    A.add(&s->page_scene, Ls >> kSlotPageShift);
    A.add(&s->usedL, 1);
    A.add(&s->usedH, 1);
    A.add(&s->wnum, 1);
    A.add(&s->ext_cnt, 4);
}

tss_status create_pool(const tss_pool_config& c, bool reserve_high, tss_solver** out) {
    if (!out) return TSS_INVALID_ARG;
    *out = nullptr;
    if (!pool_cfg_ok(c)) return TSS_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TSS_NO_DEVICE;
    tss_solver* s = new (std::nothrow) tss_solver();
    if (!s) return TSS_OOM;
    Arena A;
    PoolPlan pp;
    plan_pool(s, c, A, pp);
    s->reserve_high = reserve_high;
    std::memset(&s->cfg, 0, sizeof(s->cfg));
    s->cfg.relax_iters = c.relax_iters;
    // launch-wide parameters: capacities (the per-scene ones are in the table)
    s->P = Params{};
    s->P.relax_iters = c.relax_iters;
    s->P.slotsL = s->slotsL;
    s->P.slotsH = s->slotsH;
    s->P.capH = s->capH;
    cudaError_t e = cudaMalloc(&s->arena, A.total());
    if (e != cudaSuccess) {
        tss_status st = e == cudaErrorMemoryAllocation ? TSS_OOM : TSS_CUDA_ERROR;
        delete s;
        return st;
    }
    s->arena_bytes = A.total();
    A.carve(s->arena);
    s->L.g = grid_bufs_carve(pp.gL, s->nL, s->CL);
    s->H.g = grid_bufs_carve(pp.gH, s->capH > 0 ? s->capH : 1, s->CH);
    s->gW = grid_bufs_carve(pp.gW, s->capW > 0 ? s->capW : 1, s->CL);
    s->L.g.used = s->usedL;
    s->H.g.used = s->usedH;
    s->woff = s->gW.off;
    s->blocksL = particle_blocks(s->nL, 256);
    s->blocksH = particle_blocks(s->capH > 0 ? s->capH : 1, 256);
    s->low_full = false;
    if (tss_status la = s->apply_launch(default_launch()); la != TSS_OK) {
        delete s;
        return la;
    }
    s->ex_slots.reset(s->slotsL, TSS_POOL_SLOT_PAGE);
    s->ex_cellsL.reset(s->CL, TSS_POOL_CELL_PAGE);
    s->ex_cellsH.reset(s->CH, TSS_POOL_CELL_PAGE);
    s->ex_walls.reset(s->capW, TSS_POOL_WALL_PAGE);
    s->h_table.assign(static_cast<size_t>(c.max_scenes), Params{});
    s->h_page_scene.assign(static_cast<size_t>(s->slotsL >> kSlotPageShift), 0);
    s->scenes.assign(static_cast<size_t>(c.max_scenes), SceneRec{});
    for (int k = c.max_scenes - 1; k >= 0; --k) s->free_ids.push_back(k);
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete s;
        return TSS_CUDA_ERROR;
    }
    cudaStream_t st = s->stream;
    e = cudaMemsetAsync(s->arena, 0, A.total(), st);  // counts, grids, lists, used = 0
    if (e == cudaSuccess) launch_fill_i32(s->L.map, s->slotsL, -1, st);
    if (e == cudaSuccess) launch_fill_i32(s->H.map, s->slotsH, -1, st);
    if (e == cudaSuccess) launch_set_counts(s->cnt, 0, 0, st);
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

SceneIn scene_in(const tss_scene_desc& d) {
    return SceneIn{d.config, d.n_low, d.low_pos, d.low_vel, d.mass_low, d.mass_high, d.n_wall, d.wall_pos,
                   d.mass_wall};
}

bool scene_ok(const SceneIn& in) {
    if (!valid_cfg(in.cfg) || in.n_low < 1 || in.n_wall < 0) return false;
    if (!in.low_pos || (in.n_wall > 0 && !in.wall_pos)) return false;
    return 4LL * in.n_low < (1LL << 31) - 1;
}

// Admission checks without side effects: TSS_OK if the scene fits now.
tss_status admit_check(tss_solver* s, const SceneIn& in, tss_footprint* fp) {
    if (!scene_ok(in)) return s->fail(TSS_INVALID_ARG, "invalid scene");
    if (in.cfg->relax_iters != s->P.relax_iters)
        return s->fail(TSS_INVALID_ARG, "relax_iters differs from the pool's (one step graph for all scenes)");
    tss_footprint f;
    scene_runs(in, &f);
    const int64_t high_need = s->reserve_high ? f.high_particles : 0;
    if (!s->ex_slots.fits_ever(f.low_slots) || !s->ex_cellsL.fits_ever(f.low_cells) ||
        !s->ex_cellsH.fits_ever(f.high_cells) || !s->ex_walls.fits_ever(f.wall_particles) ||
        high_need > s->capH)
        return s->fail(TSS_INVALID_ARG, "the scene is larger than the pool");
    if (s->free_ids.empty()) return s->fail(TSS_CAPACITY, "no free scene id");
    if (s->high_reserved + high_need > s->capH) return s->fail(TSS_CAPACITY, "high-res list full");
    if (!s->ex_slots.fits_now(f.low_slots) || !s->ex_cellsL.fits_now(f.low_cells) ||
        !s->ex_cellsH.fits_now(f.high_cells) || !s->ex_walls.fits_now(f.wall_particles))
        return s->fail(TSS_CAPACITY, "no free run large enough");
    // retired scenes' entries stay in the low-res list until the next grid build
    // (an empty pool drops them at once)
    const int64_t list_low = s->n_live > 0 ? s->phys_low : 0;
    if (list_low + in.n_low > s->nL)
        return s->fail(TSS_CAPACITY, "the low-res list holds retired entries until the next step");
    if (fp) *fp = f;
    return TSS_OK;
}

tss_status admit(tss_solver* s, const SceneIn& in, cudaStream_t st, int* scene_id) {
    tss_footprint f;
    tss_status chk = admit_check(s, in, &f);
    if (chk != TSS_OK) return chk;
    const int64_t high_need = s->reserve_high ? f.high_particles : 0;
    int64_t sb = 0, cbL = 0, cbH = 0, wb = 0;
    if (!s->ex_slots.alloc(f.low_slots, &sb)) return s->fail(TSS_CAPACITY, "no free run of low-res slots");
    if (!s->ex_cellsL.alloc(f.low_cells, &cbL)) {
        s->ex_slots.release(sb);
        return s->fail(TSS_CAPACITY, "no free run of low-res cells");
    }
    if (!s->ex_cellsH.alloc(f.high_cells, &cbH)) {
        s->ex_slots.release(sb);
        s->ex_cellsL.release(cbL);
        return s->fail(TSS_CAPACITY, "no free run of high-res cells");
    }
    if (!s->ex_walls.alloc(f.wall_particles, &wb)) {
        s->ex_slots.release(sb);
        s->ex_cellsL.release(cbL);
        s->ex_cellsH.release(cbH);
        return s->fail(TSS_CAPACITY, "no free run of wall particles");
    }
    cudaError_t e0 = cudaSuccess;
    if (s->n_live == 0 && s->phys_low > 0) {  // only retired entries left: drop them now
        launch_set_counts(s->cnt, 0, 0, st);
        s->phys_low = 0;
        e0 = cudaGetLastError();
    }
    const int id = s->free_ids.back();
    s->free_ids.pop_back();
    Params P = make_params(in);
    P.cbL = static_cast<int>(cbL);
    P.cbH = static_cast<int>(cbH);
    P.sbL = static_cast<int>(sb);
    P.wb = static_cast<int>(wb);
    P.slotsL = s->slotsL;
    P.slotsH = s->slotsH;
    P.capH = s->capH;
    P.step0 = s->steps_issued;  // the scene's ROI motion starts at its first step
    s->h_table[id] = P;
    const int n = in.n_low, nW = in.n_wall;
    const int base = static_cast<int>(s->phys_low);
    const int CLs = in.cfg->dims_low[0] * in.cfg->dims_low[1];
    const int64_t p0 = sb >> kSlotPageShift, np = s->ex_slots.pages(n);
    for (int64_t p = p0; p < p0 + np; ++p) s->h_page_scene[static_cast<size_t>(p)] = static_cast<uint16_t>(id);

    // Host arrays: the pageable ones are staged by the copy calls before they return.
    cudaError_t e = e0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_table + id, &s->h_table[id], sizeof(Params), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->page_scene + p0, s->h_page_scene.data() + p0, sizeof(uint16_t) * np,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->L.npos + base, in.low_pos, sizeof(float2) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = in.low_vel ? cudaMemcpyAsync(s->L.nvel + base, in.low_vel, sizeof(float2) * n, cudaMemcpyHostToDevice, st)
                       : cudaMemsetAsync(s->L.nvel + base, 0, sizeof(float2) * n, st);
    if (e == cudaSuccess) {
        k_admit_low<<<particle_blocks(n, 256), 256, 0, st>>>(s->L.npos, s->L.nid, s->L.nst,
                                                             s->carry ? s->L.ndens : nullptr, s->L.npres, base, n,
                                                             static_cast<int>(sb), P, s->L.g);
        launch_fill_i32(s->H.map + 4 * sb, 4LL * n, -1, st);
        k_set_int<<<1, 1, 0, st>>>(&s->cnt->cur[0], base + n);
        e = cudaGetLastError();
    }
    // the scene's wall grid: (cell, id) order within the scene, scene-local offsets
    if (e == cudaSuccess && nW > 0) {
        e = cudaMemcpyAsync(s->wraw + wb, in.wall_pos, sizeof(float2) * nW, cudaMemcpyHostToDevice, st);
        launch_iota(s->wid + wb, nW, st);
        k_set_int<<<1, 1, 0, st>>>(s->wnum, nW);
        GridBufs gv = s->gW;
        gv.ncells = CLs;
        gv.ntiles = (CLs + kScanTile - 1) / kScanTile;
        gv.count = s->gW.count + cbL;
        gv.off = s->woff + cbL;
        gv.key = s->gW.key + wb;
        gv.rank = s->gW.rank + wb;
        gv.perm = s->gW.perm + wb;
        gv.used = nullptr;
        ReorderArgs a{};
        a.src_pos = s->wraw + wb;
        a.dst_pos = s->wpos + wb;
        if (e == cudaSuccess)
            e = grid_build_enqueue(s->wraw + wb, s->wid + wb, s->wnum, nW, P.ox, P.oy, P.r, P.dimL[0], P.dimL[1], gv, a,
                                   &s->cnt->err, st);
    } else if (e == cudaSuccess) {
        e = cudaMemsetAsync(s->woff + cbL, 0, sizeof(int) * (static_cast<size_t>(CLs) + 1), st);
    }
    if (e == cudaSuccess) launch_wall_near(s->woff + cbL, s->wnear + cbL, P.dimL[0], P.dimL[1], st);
    if (e == cudaSuccess) {
        k_set_int<<<1, 1, 0, st>>>(s->usedL, static_cast<int>(s->ex_cellsL.high_water()));
        k_set_int<<<1, 1, 0, st>>>(s->usedH, static_cast<int>(s->ex_cellsH.high_water()));
        e = cudaGetLastError();
    }
    SceneRec& r = s->scenes[id];
    r.live = true;
    r.sb = sb;
    r.n_low = n;
    r.cbL = cbL;
    r.nCL = f.low_cells;
    r.cbH = cbH;
    r.nCH = f.high_cells;
    r.wb = wb;
    r.nW = nW;
    r.high_res = high_need;
    r.admitted_step = s->steps_issued;
    s->high_reserved += high_need;
    s->phys_low += n;
    s->live_low += n;
    ++s->n_live;
    *scene_id = id;
    if (e != cudaSuccess) return s->cuda_fail(e, "admit");
    return TSS_OK;
}

}  // namespace

extern "C" {

tss_status tss_scene_footprint(const tss_scene_desc* scene, tss_footprint* out) {
    if (!scene || !out) return TSS_INVALID_ARG;
    const SceneIn in = scene_in(*scene);
    if (!scene_ok(in)) return TSS_INVALID_ARG;
    tss_footprint f;
    scene_runs(in, &f);
    auto rnd = [](int64_t n, int64_t p) { return (n + p - 1) / p * p; };
    out->low_slots = rnd(f.low_slots, TSS_POOL_SLOT_PAGE);
    out->high_particles = f.high_particles;
    out->low_cells = rnd(f.low_cells, TSS_POOL_CELL_PAGE);
    out->high_cells = rnd(f.high_cells, TSS_POOL_CELL_PAGE);
    out->wall_particles = rnd(f.wall_particles, TSS_POOL_WALL_PAGE);
    return TSS_OK;
}

tss_status tss_pool_bytes(const tss_pool_config* cfg, size_t* bytes) {
    if (!cfg || !bytes || !pool_cfg_ok(*cfg)) return TSS_INVALID_ARG;
    tss_solver tmp;  // sizing only: no device memory, stream or graph is created
    Arena A;
    PoolPlan pp;
    plan_pool(&tmp, *cfg, A, pp);
    *bytes = A.total();
    return TSS_OK;
}

tss_status tss_pool_config_for_budget(size_t bytes, double low_cells_per_slot, double walls_per_slot,
                                      int max_scenes, int relax_iters, tss_pool_config* out) {
    if (!out || !(low_cells_per_slot > 0) || !(walls_per_slot >= 0) || max_scenes < 1 ||
        max_scenes > TSS_POOL_MAX_SCENES || relax_iters < 0)
        return TSS_INVALID_ARG;
    auto make = [&](int64_t slots) {
        tss_pool_config c{};
        c.low_slots = std::max<int64_t>(slots, TSS_POOL_SLOT_PAGE);
        c.high_particles = 4 * c.low_slots;
        c.low_cells = std::max<int64_t>(static_cast<int64_t>(low_cells_per_slot * c.low_slots), TSS_POOL_CELL_PAGE);
        c.high_cells = std::max<int64_t>(4 * c.low_cells, TSS_POOL_CELL_PAGE);
        c.wall_particles = static_cast<int64_t>(walls_per_slot * c.low_slots);
        c.max_scenes = max_scenes;
        c.relax_iters = relax_iters;
        return c;
    };
    // bytes are affine in the slots: size two pools and solve, then step down to fit
    size_t b0 = 0, b1 = 0;
    const int64_t s0 = 1 << 16, s1 = 1 << 20;
    tss_pool_config c0 = make(s0), c1 = make(s1);
    if (tss_pool_bytes(&c0, &b0) != TSS_OK || tss_pool_bytes(&c1, &b1) != TSS_OK) return TSS_INVALID_ARG;
    const double per = static_cast<double>(b1 - b0) / static_cast<double>(s1 - s0);
    const double fixed = static_cast<double>(b0) - per * s0;
    if (static_cast<double>(bytes) <= fixed + per * TSS_POOL_SLOT_PAGE) return TSS_INVALID_ARG;
    int64_t slots = static_cast<int64_t>((static_cast<double>(bytes) - fixed) / per);
    // int32 limits of the slot, list and cell spaces
    const int64_t lim = std::min<int64_t>({1LL << 29, ((1LL << 31) - 2) / 4,
                                           static_cast<int64_t>(((1LL << 31) - 2) / (4.0 * low_cells_per_slot))});
    slots = std::min(slots, lim);
    slots = slots / TSS_POOL_SLOT_PAGE * TSS_POOL_SLOT_PAGE;
    for (;;) {
        tss_pool_config c = make(slots);
        size_t b = 0;
        if (tss_pool_bytes(&c, &b) != TSS_OK) return TSS_INVALID_ARG;
        if (b <= bytes) {
            *out = c;
            return TSS_OK;
        }
        slots -= std::max<int64_t>(TSS_POOL_SLOT_PAGE, slots / 1000 / TSS_POOL_SLOT_PAGE * TSS_POOL_SLOT_PAGE);
        if (slots < TSS_POOL_SLOT_PAGE) return TSS_INVALID_ARG;
    }
}

tss_status tss_pool_create(const tss_pool_config* cfg, tss_solver** out) {
    if (!cfg) return TSS_INVALID_ARG;
    return create_pool(*cfg, true, out);
}

tss_status tss_pool_admit(tss_solver* s, const tss_scene_desc* scene, void* stream, int* scene_id) {
    if (!s || !scene || !scene_id || !s->batched) return TSS_INVALID_ARG;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = s->enter(st);
    if (e != cudaSuccess) return s->cuda_fail(e, "admit");
    const tss_status r = admit(s, scene_in(*scene), st, scene_id);
    if ((e = s->leave(st)) != cudaSuccess) return s->cuda_fail(e, "admit");
    return r;
}

tss_status tss_pool_can_admit(tss_solver* s, const tss_scene_desc* scene) {
    if (!s || !scene || !s->batched) return TSS_INVALID_ARG;
    return admit_check(s, scene_in(*scene), nullptr);
}

tss_status tss_pool_retire(tss_solver* s, int id, void* stream) {
    if (!s || !s->batched || id < 0 || id >= s->S || !s->scenes[id].live) return TSS_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = s->enter(st);
    if (e != cudaSuccess) return s->cuda_fail(e, "retire");
    SceneRec& r = s->scenes[id];
    const int lo = static_cast<int>(r.sb), hi = static_cast<int>(r.sb + r.n_low);
    k_retire<<<s->blocksL, 256, 0, st>>>(s->L.nid, &s->cnt->cur[0], s->nL, 0, lo, hi, s->L.g, nullptr, 0);
    k_retire<<<s->blocksH, 256, 0, st>>>(s->H.nid, &s->cnt->cur[1], s->capH, 2, lo, hi, s->H.g, s->H.map,
                                         s->slotsH);
    s->ex_slots.release(r.sb);
    s->ex_cellsL.release(r.cbL);
    s->ex_cellsH.release(r.cbH);
    if (r.nW > 0) s->ex_walls.release(r.wb);
    k_set_int<<<1, 1, 0, st>>>(s->usedL, static_cast<int>(s->ex_cellsL.high_water()));
    k_set_int<<<1, 1, 0, st>>>(s->usedH, static_cast<int>(s->ex_cellsH.high_water()));
    s->high_reserved -= r.high_res;
    s->live_low -= r.n_low;
    --s->n_live;
    r.live = false;
    s->free_ids.push_back(id);
    std::sort(s->free_ids.begin(), s->free_ids.end(), std::greater<int>());  // lowest id on top
    e = cudaGetLastError();
    if (e == cudaSuccess) e = s->leave(st);
    if (e != cudaSuccess) return s->cuda_fail(e, "retire");
    return TSS_OK;
}

tss_status tss_pool_free(tss_solver* s, tss_footprint* f) {
    if (!s || !f || !s->batched) return TSS_INVALID_ARG;
    f->low_slots = s->ex_slots.free_units();
    f->high_particles = s->capH - s->high_reserved;
    f->low_cells = s->ex_cellsL.free_units();
    f->high_cells = s->ex_cellsH.free_units();
    f->wall_particles = s->ex_walls.free_units();
    return TSS_OK;
}

tss_status tss_pool_extract(tss_solver* s, int id, const tss_scene_result* dst, int32_t* d_counts, void* stream) {
    if (!s || !s->batched || !dst || !d_counts || id < 0 || id >= s->S || !s->scenes[id].live)
        return TSS_INVALID_ARG;
    const SceneRec& r = s->scenes[id];
    if (s->steps_issued <= r.admitted_step) return s->fail(TSS_INVALID_ARG, "the scene has not taken a step");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Params& P = s->h_table[id];
    const int CLs = P.dimL[0] * P.dimL[1];
    cudaError_t e = s->enter(st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->ext_cnt, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return s->cuda_fail(e, "extract");
    k_count_splits<<<particle_blocks(static_cast<int>(std::max<int64_t>(s->live_low, 1)), 256), 256, 0, st>>>(
        s->split_flag, s->L.g.off, P.cbL, CLs, s->cnt, s->ext_cnt, d_counts);
    ExtractArgs a{};
    a.sb = P.sbL;
    a.n_low = static_cast<int>(r.n_low);
    a.cbL = P.cbL;
    a.CLs = CLs;
    a.cbH = P.cbH;
    a.CHs = P.CHs;
    a.lpos = s->L.npos;
    a.lvel = s->L.nvel;
    a.hpos = s->H.npos;
    a.hvel = s->H.nvel;
    a.lst = s->L.nst;
    a.hst = s->H.nst;
    a.lid = s->L.nid;
    a.hid = s->H.nid;
    a.ldens = s->carry ? s->L.ndens : s->L.dens;
    a.lpres = s->carry ? s->L.npres : s->L.pres;
    a.hdens = s->carry ? s->H.ndens : s->H.dens;
    a.hpres = s->carry ? s->H.npres : s->H.pres;
    a.kid_dens = s->carry;
    a.offL = s->L.g.off;
    a.offH = s->H.g.off;
    a.cnt = s->cnt;
    a.splits = s->ext_cnt;
    a.dst = *dst;
    a.d_counts = d_counts;
    k_extract<<<particle_blocks(static_cast<int>(std::min<int64_t>(5 * r.n_low, 1 << 30)), 256), 256, 0, st>>>(a);
    if ((e = cudaGetLastError()) == cudaSuccess) e = s->leave(st);
    if (e != cudaSuccess) return s->cuda_fail(e, "extract");
    return TSS_OK;
}

// A batch: a pool sized for exactly these scenes; scene k is admitted as scene k.
tss_status tss_batch_create(int n_scenes, const tss_scene_desc* scenes, int cap_high, tss_solver** out) {
    if (!out || !scenes || n_scenes < 1 || n_scenes > TSS_POOL_MAX_SCENES || cap_high < 0) return TSS_INVALID_ARG;
    *out = nullptr;
    tss_pool_config c{};
    for (int k = 0; k < n_scenes; ++k) {
        const SceneIn in = scene_in(scenes[k]);
        if (!scene_ok(in) || in.cfg->relax_iters != scenes[0].config->relax_iters) return TSS_INVALID_ARG;
        tss_footprint f;
        if (tss_scene_footprint(&scenes[k], &f) != TSS_OK) return TSS_INVALID_ARG;
        c.low_slots += f.low_slots;
        c.low_cells += f.low_cells;
        c.high_cells += f.high_cells;
        c.wall_particles += f.wall_particles;
    }
    c.low_cells = std::max<int64_t>(c.low_cells, TSS_POOL_CELL_PAGE);
    c.high_cells = std::max<int64_t>(c.high_cells, TSS_POOL_CELL_PAGE);
    c.high_particles = cap_high;
    c.max_scenes = n_scenes;
    c.relax_iters = scenes[0].config->relax_iters;
    if (!pool_cfg_ok(c)) return TSS_INVALID_ARG;
    tss_solver* s = nullptr;
    tss_status st = create_pool(c, false, &s);
    if (st != TSS_OK) return st;
    s->blocksL = (s->nL + 255) / 256;  // the low-res list is full: one block per 256 particles
    s->low_full = true;
    if ((st = s->apply_launch(default_launch())) != TSS_OK) {
        delete s;
        return st;
    }
    // ids are handed out lowest first, so scene k gets id k
    for (int k = 0; k < n_scenes; ++k) {
        int id = -1;
        st = admit(s, scene_in(scenes[k]), s->stream, &id);
        if (st != TSS_OK || id != k) {
            delete s;
            return st != TSS_OK ? st : TSS_CUDA_ERROR;
        }
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        delete s;
        return TSS_CUDA_ERROR;
    }
    *out = s;
    return TSS_OK;
}

tss_status tss_solver_num_scenes(tss_solver* s, int* n) {
    if (!s || !n) return TSS_INVALID_ARG;
    if (!s->batched) {
        *n = 1;
        return TSS_OK;
    }
    int top = 0;
    for (int k = 0; k < s->S; ++k)
        if (s->scenes[k].live) top = k + 1;
    *n = top;
    return TSS_OK;
}

tss_status tss_solver_scene_counts(tss_solver* s, int* n_low, int* n_high) {
    if (!s) return TSS_INVALID_ARG;
    int ns = 0;
    tss_solver_num_scenes(s, &ns);
    tss_counts c;
    tss_status st = tss_solver_counts(s, &c);
    if (st != TSS_OK) return st;
    if (!s->batched) {
        if (n_low) n_low[0] = c.n_low;
        if (n_high) n_high[0] = c.n_high;
        return TSS_OK;
    }
    if (n_low)
        for (int k = 0; k < ns; ++k) n_low[k] = s->scenes[k].live ? static_cast<int>(s->scenes[k].n_low) : 0;
    if (n_high) {
        std::vector<int32_t> ids(static_cast<size_t>(c.n_high));
        cudaError_t e = c.n_high ? s->d2h(ids.data(), s->H.nid, sizeof(int32_t) * c.n_high)
                                 : cudaSuccess;
        if (e != cudaSuccess) return s->cuda_fail(e, "scene counts");
        for (int k = 0; k < ns; ++k) n_high[k] = 0;
        for (int32_t id : ids) {
            const int low = id >> 2;
            if (low < 0 || low >= s->slotsL) continue;
            const int k = s->h_page_scene[static_cast<size_t>(low) >> kSlotPageShift];
            const SceneRec& r = s->scenes[k];
            if (k < ns && r.live && low >= r.sb && low < r.sb + r.n_low) ++n_high[k];
        }
    }
    return TSS_OK;
}

tss_status tss_solver_download_scene(tss_solver* s, int scene, int scale, tss_scale_state* out) {
    if (!s || !out || (scale != 0 && scale != 1)) return TSS_INVALID_ARG;
    if (!s->batched) return scene == 0 ? tss_solver_download(s, scale, out) : TSS_INVALID_ARG;
    if (scene < 0 || scene >= s->S || !s->scenes[scene].live) return TSS_INVALID_ARG;
    tss_counts c;
    tss_status st = tss_solver_counts(s, &c);
    if (st != TSS_OK) return st;
    const int n = scale == 0 ? c.n_low : c.n_high;
    std::vector<int32_t> id(n);
    std::vector<float> pos(2 * static_cast<size_t>(n)), vel(2 * static_cast<size_t>(n)), dens(n), pres(n);
    std::vector<uint8_t> stt(n);
    tss_scale_state all{n, id.data(), pos.data(), vel.data(), stt.data(), dens.data(), pres.data()};
    if ((st = tss_solver_download(s, scale, &all)) != TSS_OK) return st;
    const int shift = scale == 0 ? 0 : 2;
    const SceneRec& r = s->scenes[scene];
    const int64_t lo = r.sb, hi = r.sb + r.n_low;
    int m = 0;
    for (int i = 0; i < n; ++i) {
        const int low = id[i] >> shift;
        if (low < lo || low >= hi) continue;
        if (m < out->n) {
            if (out->id) out->id[m] = id[i] - static_cast<int32_t>(lo << shift);
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
        }
        ++m;
    }
    const bool fits = m <= out->n;
    out->n = m;
    return fits ? TSS_OK : s->fail(TSS_INVALID_ARG, "download buffer too small");
}

}  // extern "C"
