// refgpu_launcher.cu -- runs the reference's own CUDA kernels, rebuilt for sm_103a
// (oracle/_ref/refkern.cubin, see build_refgpu.sh), on the GPU, headless.  ORACLE /
// MEASUREMENT INFRASTRUCTURE ONLY: it times the reference beside this library and
// gives a second, approximate result source; nothing of the library uses it.
//
// This restates the host side of WCSPHSolver (TwoScale2D/WCSPHSolver.cu:2343-3238)
// without OpenGL: the particle systems are plain device arrays (ParticleSystem's
// VBOs), the constants are set as Bind() sets them (2537-2639), the boundary grid
// is built as initBoundaries() builds it (3205-3238), and each step issues what
// AdvanceTS issues (2726-2810): the two neighbour-grid updates with their full-table
// clears and thrust::sort_by_key, the density, acceleration and integration kernels
// with the reference's launch shapes (256-thread blocks, ceil(n/256) blocks), the
// transient adjustment, and the three synchronous count read-backs.  The visual
// quantities for the renderer (setVisualQuantities) are not computed: rendering is
// not part of the step here.  The reference's schedule is the GPU's own (atomic
// list appends, in-place integration), as in the reference.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/sort.h>

#include "tss.h"

namespace {

constexpr double kRefPi = 3.14159265358979323846;  // WCSPHSolver.cu:19 (a double literal)
constexpr unsigned kBlock = 256;                    // mBlockDim (WCSPHSolver.cu:2421,2437)

enum Fn {
    kInitIds, kHash, kHashHigh, kCellRanges, kDensity, kDensityHigh, kAccel, kAccelHigh, kAdvance, kAdjust, kNumFn
};
const char* const kFnName[kNumFn] = {
    "ref_initParticleIDs",  "ref_computeParticleHash",         "ref_computeParticleHashHigh",
    "ref_computeCellStartEndIndices", "ref_computeParticleDensityPressure",
    "ref_computeParticleDensityPressureHigh", "ref_computeParticleAcceleration",
    "ref_computeParticleAccelerationAndAdvanceHigh", "ref_advance", "ref_adjustOrInjectTransientHighD"};

struct Sys {  // one ParticleSystem (ParticleSystem.h:17-78), slot-indexed device arrays
    int num = 0, max = 0;
    float mass = 0.f;
    float *pos = nullptr, *vel = nullptr, *acc = nullptr, *dens = nullptr, *pres = nullptr, *vis = nullptr;
    int* gl = nullptr;  // the GL index buffer the kernels maintain
};

struct Grid {  // NeighborGrid (WCSPHSolver.cu:2343-2389)
    int cells = 0;
    int *hash = nullptr, *start = nullptr, *end = nullptr, *ids[2] = {nullptr, nullptr};
};

struct RefGpu {
    CUmodule mod = nullptr;
    CUfunction fn[kNumFn] = {};
    tss_config cfg{};
    Sys L, H, B;
    Grid gL, gH;
    unsigned char *stL = nullptr, *stH = nullptr;
    int* trL[2] = {nullptr, nullptr};
    int *cntL = nullptr, *cntH = nullptr, *cntTrL = nullptr;  // device counters
    int nTrL = 0;                                            // mTransientParticleCountLow
    int active = 0;                                          // activeID
    int *bHash = nullptr, *bIds = nullptr, *bStart = nullptr, *bEnd = nullptr;
    std::vector<void*> allocs;
    std::string err;
    long long steps = 0;

    ~RefGpu() {
        for (void* p : allocs) cudaFree(p);
        if (mod) cuModuleUnload(mod);
    }

    template <class T>
    bool alloc(T** p, size_t count) {
        void* q = nullptr;
        if (cudaMalloc(&q, sizeof(T) * (count ? count : 1)) != cudaSuccess) return fail("cudaMalloc");
        allocs.push_back(q);
        *p = static_cast<T*>(q);
        return true;
    }
    bool fail(const std::string& what) {
        if (err.empty()) err = what;
        return false;
    }
    bool cu(CUresult r, const char* what) {
        if (r == CUDA_SUCCESS) return true;
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        return fail(std::string(what) + ": " + (s ? s : "?"));
    }
    bool rt(cudaError_t e, const char* what) {
        return e == cudaSuccess ? true : fail(std::string(what) + ": " + cudaGetErrorString(e));
    }

    // kernel<<<ceil(n/256), 256, shmem>>>(args...) on the default stream
    bool launch(Fn f, unsigned n, unsigned shmem, void** args) {
        if (n == 0) return true;
        const unsigned blocks = (n + kBlock - 1) / kBlock;
        return cu(cuLaunchKernel(fn[f], blocks, 1, 1, kBlock, 1, 1, shmem, nullptr, args, nullptr), kFnName[f]);
    }

    template <class T>
    bool set_symbol(const char* name, const T* v, size_t count) {
        CUdeviceptr p = 0;
        size_t bytes = 0;
        if (!cu(cuModuleGetGlobal(&p, &bytes, mod, name), name)) return false;
        if (bytes != sizeof(T) * count) return fail(std::string("size of ") + name);
        return cu(cuMemcpyHtoD(p, v, bytes), name);
    }

    bool set_texture(const char* name, const void* ptr, int n) {
        struct {
            const void* ptr;
            int n;
        } t{ptr, n};
        CUdeviceptr p = 0;
        size_t bytes = 0;
        if (!cu(cuModuleGetGlobal(&p, &bytes, mod, name), name)) return false;
        if (bytes != sizeof(t)) return fail(std::string("layout of ") + name);
        return cu(cuMemcpyHtoD(p, &t, sizeof(t)), name);
    }

    bool sort_by_key(int* keys, int* vals, int n) {  // thrust::sort_by_key as the reference calls it
        if (n <= 0) return true;
        thrust::sort_by_key(thrust::device_ptr<int>(keys), thrust::device_ptr<int>(keys + n),
                            thrust::device_ptr<int>(vals));
        return rt(cudaGetLastError(), "sort_by_key");
    }

    bool cell_ranges(int* start, int* end, int* hash, int n) {  // computeCellStartEndIndices
        unsigned un = static_cast<unsigned>(n);
        void* a[] = {&start, &end, &hash, &un};
        return launch(kCellRanges, un, sizeof(int) * (kBlock + 1), a);
    }

    bool bind() {  // Bind(), WCSPHSolver.cu:2537-2639
        const float r = cfg.r_low, rh = cfg.r_high;
        const float coeff = 20.0f / (14.0f * kRefPi * r * r);
        const float grad = -120.0f / (14.0f * kRefPi * r * r * r);
        const float coeffH = 20.0f / (14.0f * kRefPi * rh * rh);
        const float gradH = -120.0f / (14.0f * kRefPi * rh * rh * rh);
        return set_symbol("gdDomainOrigin", cfg.domain_origin, 2) &&
               set_symbol("gdDomainDimensions", cfg.dims_low, 2) &&
               set_symbol("gdDomainDimensionsHigh", cfg.dims_high, 2) &&
               set_symbol("gdEffectiveRadius", &cfg.r_low, 1) && set_symbol("gdEffectiveRadiusHigh", &cfg.r_high, 1) &&
               set_symbol("gdRestDensity", &cfg.rest_density, 1) && set_symbol("gdTaitCoefficient", &cfg.tait_b, 1) &&
               set_symbol("gdSpeedSound", &cfg.speed_sound, 1) && set_symbol("gdAlpha", &cfg.alpha, 1) &&
               set_symbol("gdTensionCoefficient", &cfg.tension, 1) && set_symbol("gdM4KernelCoeff", &coeff, 1) &&
               set_symbol("gdM4KernelGradCoeff", &grad, 1) && set_symbol("gdM4KernelCoeffHigh", &coeffH, 1) &&
               set_symbol("gdM4KernelGradCoeffHigh", &gradH, 1) &&
               set_symbol("gdFluidParticleMass", &L.mass, 1) && set_symbol("gdFluidParticleMassHigh", &H.mass, 1) &&
               set_symbol("gdBoundaryParticleMass", &B.mass, 1);
    }

    bool init_boundaries() {  // initBoundaries(), WCSPHSolver.cu:3205-3238, and the texture binds
        const int n = B.num;
        const int cells = gL.cells;
        unsigned un = static_cast<unsigned>(n);
        void* a0[] = {&bIds, &un};
        if (!launch(kInitIds, un, 0, a0)) return false;
        void* a1[] = {&bHash, &bIds, &B.pos, &un};
        if (!launch(kHash, un, 0, a1)) return false;
        if (!sort_by_key(bHash, bIds, n)) return false;
        if (!rt(cudaMemset(bStart, 0xFF, sizeof(int) * cells), "memset") ||
            !rt(cudaMemset(bEnd, 0xFF, sizeof(int) * cells), "memset"))
            return false;
        if (!cell_ranges(bStart, bEnd, bHash, n)) return false;
        return set_texture("gdBoundaryPositionsTex", B.pos, 2 * n) &&
               set_texture("gdBoundaryParticleIDsTex", bIds, n) &&
               set_texture("gdBoundaryCellStartIndicesTex", bStart, cells) &&
               set_texture("gdBoundaryCellEndIndicesTex", bEnd, cells);
    }

    bool grid_high(int a) {  // updateNeighborGridHigh, WCSPHSolver.cu:2934-2979
        if (!rt(cudaMemset(gH.start, 0xFF, sizeof(int) * gH.cells), "memset") ||
            !rt(cudaMemset(gH.end, 0xFF, sizeof(int) * gH.cells), "memset"))
            return false;
        if (H.num == 0) return true;
        unsigned n = static_cast<unsigned>(H.num);
        int* ids = gH.ids[a];
        void* args[] = {&gH.hash, &ids, &H.pos, &n};
        return launch(kHashHigh, n, 0, args) && sort_by_key(gH.hash, ids, H.num) &&
               cell_ranges(gH.start, gH.end, gH.hash, H.num);
    }

    bool grid_low(int a) {  // updateNeighborGrid, WCSPHSolver.cu:2814-2854
        unsigned n = static_cast<unsigned>(L.num);
        int* ids = gL.ids[a];
        void* args[] = {&gL.hash, &ids, &L.pos, &n};
        return launch(kHash, n, 0, args) && sort_by_key(gL.hash, ids, L.num) &&
               rt(cudaMemset(gL.start, 0xFF, sizeof(int) * gL.cells), "memset") &&
               rt(cudaMemset(gL.end, 0xFF, sizeof(int) * gL.cells), "memset") &&
               cell_ranges(gL.start, gL.end, gL.hash, L.num);
    }

    bool step() {  // AdvanceTS, WCSPHSolver.cu:2726-2810
        const int a = active, b = 1 - a;
        if (!grid_high(a) || !grid_low(a)) return false;
        float dt = cfg.dt;
        unsigned nL = static_cast<unsigned>(L.num), nH = static_cast<unsigned>(H.num);
        int *idsLa = gL.ids[a], *idsLb = gL.ids[b], *idsHa = gH.ids[a], *idsHb = gH.ids[b];
        if (nH > 0) {  // computePressureDensityHigh, 3019-3042
            void* args[] = {&H.dens, &H.pres, &idsHa, &gH.start, &gH.end, &H.pos, &stH,
                            &idsLa,  &gL.start, &gL.end, &L.pos, &stL, &nH};
            if (!launch(kDensityHigh, nH, 0, args)) return false;
        }
        {  // computePressureDensity, 2856-2874
            void* args[] = {&L.dens, &L.pres, &idsLa, &gL.start, &gL.end, &L.pos, &stL,
                            &idsHa,  &gH.start, &gH.end, &H.pos, &stH, &nL};
            if (!launch(kDensity, nL, 0, args)) return false;
        }
        // computeAccelerations, 2876-2919
        if (!rt(cudaMemset(cntL, 0, sizeof(int)), "memset") || !rt(cudaMemset(cntTrL, 0, sizeof(int)), "memset") ||
            !rt(cudaMemset(cntH, 0, sizeof(int)), "memset"))
            return false;
        {
            int* trb = trL[b];
            void* args[] = {&L.acc,  &L.vis,  &L.pos,  &L.vel,   &stL,      &stH,    &idsLb,  &idsHb, &L.gl, &H.gl,
                            &trb,    &cntL,   &cntH,   &cntTrL,  &L.dens,   &L.pres, &H.pos,  &H.vel, &H.dens,
                            &H.pres, &idsLa,  &gL.start, &gL.end, &idsHa,   &gH.start, &gH.end, &dt, &nL};
            if (!launch(kAccel, nL, 0, args)) return false;
        }
        if (nH > 0) {  // updatePositionsHigh, 2981-3017
            void* args[] = {&H.pos,  &H.vel,  &H.acc,  &idsHb,   &H.gl,    &cntH,   &H.dens, &H.pres,
                            &stH,    &L.pos,  &L.vel,  &L.dens,  &L.pres,  &stL,    &idsHa,  &gH.start,
                            &gH.end, &idsLa,  &gL.start, &gL.end, &dt,     &nH};
            if (!launch(kAccelHigh, nH, 0, args)) return false;
        }
        {  // updatePositions, 2921-2932
            void* args[] = {&L.pos, &L.vel, &L.acc, &idsLa, &dt, &nL};
            if (!launch(kAdvance, nL, 0, args)) return false;
        }
        if (nTrL > 0) {  // adjustOrInjectTransientHigh, 3112-3139
            unsigned nt = static_cast<unsigned>(nTrL);
            int *tra = trL[a], *trb = trL[b];
            void* args[] = {&H.pos, &H.vel, &stH, &idsLb, &L.gl, &trb, &cntL, &cntTrL, &L.pos, &L.vel, &L.dens,
                            &tra,   &nt};
            if (!launch(kAdjust, nt, 0, args)) return false;
        }
        // the count read-backs (2760-2781): synchronous copies, as in the reference
        if (!rt(cudaMemcpy(&L.num, cntL, sizeof(int), cudaMemcpyDeviceToHost), "count") ||
            !rt(cudaMemcpy(&H.num, cntH, sizeof(int), cudaMemcpyDeviceToHost), "count") ||
            !rt(cudaMemcpy(&nTrL, cntTrL, sizeof(int), cudaMemcpyDeviceToHost), "count"))
            return false;
        if (L.num < 0 || L.num > L.max || H.num < 0 || H.num > H.max || nTrL < 0 || nTrL > L.max)
            return fail("a particle count left its capacity");
        active = b;
        ++steps;
        return true;
    }

    // Replaces the particle state with a state taken elsewhere (a developed scene),
    // kept as the reference keeps it: slot-indexed arrays, the active low id list
    // holding every low-res slot (split parents stay in it), the active high id
    // list the given high-res slots, and the active transient list every split
    // parent (each step re-appends them, WCSPHSolver.cu:1135-1140).  low_* have
    // L.max entries by slot; high_* are in list order.
    bool set_state(const float* low_pos, const float* low_vel, const unsigned char* low_st, int n_high,
                   const int* high_ids, const float* high_pos, const float* high_vel, const unsigned char* high_st) {
        if (n_high < 0 || n_high > H.max) return fail("set_state: high-res count out of range");
        const size_t nl = static_cast<size_t>(L.max), nh = static_cast<size_t>(H.max);
        std::vector<float> hp(2 * nh, 0.0f), hv(2 * nh, 0.0f);
        std::vector<unsigned char> hs(nh, 0);
        std::vector<int> tr;
        for (int k = 0; k < n_high; ++k) {
            const int id = high_ids[k];
            if (id < 0 || id >= H.max) return fail("set_state: high-res id out of range");
            hp[2 * id] = high_pos[2 * k];
            hp[2 * id + 1] = high_pos[2 * k + 1];
            hv[2 * id] = high_vel[2 * k];
            hv[2 * id + 1] = high_vel[2 * k + 1];
            hs[id] = high_st[k];
        }
        for (int i = 0; i < L.max; ++i)
            if (low_st[i] == 1) tr.push_back(i);
        std::vector<int> lid(nl);
        for (int i = 0; i < L.max; ++i) lid[i] = i;
        const int a = active;
        bool ok = rt(cudaMemcpy(L.pos, low_pos, sizeof(float) * 2 * nl, cudaMemcpyHostToDevice), "set_state") &&
                  rt(cudaMemcpy(L.vel, low_vel, sizeof(float) * 2 * nl, cudaMemcpyHostToDevice), "set_state") &&
                  rt(cudaMemcpy(stL, low_st, nl, cudaMemcpyHostToDevice), "set_state") &&
                  rt(cudaMemcpy(gL.ids[a], lid.data(), sizeof(int) * nl, cudaMemcpyHostToDevice), "set_state") &&
                  rt(cudaMemcpy(H.pos, hp.data(), sizeof(float) * 2 * nh, cudaMemcpyHostToDevice), "set_state") &&
                  rt(cudaMemcpy(H.vel, hv.data(), sizeof(float) * 2 * nh, cudaMemcpyHostToDevice), "set_state") &&
                  rt(cudaMemcpy(stH, hs.data(), nh, cudaMemcpyHostToDevice), "set_state");
        if (ok && n_high > 0)
            ok = rt(cudaMemcpy(gH.ids[a], high_ids, sizeof(int) * n_high, cudaMemcpyHostToDevice), "set_state");
        if (ok && !tr.empty())
            ok = rt(cudaMemcpy(trL[a], tr.data(), sizeof(int) * tr.size(), cudaMemcpyHostToDevice), "set_state");
        if (!ok) return false;
        L.num = L.max;
        H.num = n_high;
        nTrL = static_cast<int>(tr.size());
        return rt(cudaDeviceSynchronize(), "set_state");
    }

    bool create(const char* cubin, const tss_config* c, int n_low, const float* low_pos, const float* low_vel,
                float mass_low, int cap_high, float mass_high, int n_wall, const float* wall_pos, float mass_wall) {
        cfg = *c;
        if (!rt(cudaFree(nullptr), "context")) return false;  // the runtime's primary context, current
        if (!cu(cuModuleLoad(&mod, cubin), cubin)) return false;
        for (int f = 0; f < kNumFn; ++f)
            if (!cu(cuModuleGetFunction(&fn[f], mod, kFnName[f]), kFnName[f])) return false;
        L.max = n_low;
        L.num = n_low;
        L.mass = mass_low;
        H.max = cap_high;
        H.mass = mass_high;
        B.max = B.num = n_wall;
        B.mass = mass_wall;
        gL.cells = cfg.dims_low[0] * cfg.dims_low[1];
        gH.cells = cfg.dims_high[0] * cfg.dims_high[1];
        for (Sys* s : {&L, &H, &B}) {
            const size_t m = static_cast<size_t>(s->max);
            if (!alloc(&s->pos, 2 * m) || !alloc(&s->vel, 2 * m) || !alloc(&s->acc, 2 * m) || !alloc(&s->dens, m) ||
                !alloc(&s->pres, m) || !alloc(&s->vis, m) || !alloc(&s->gl, m))
                return false;
            if (!rt(cudaMemset(s->pos, 0, sizeof(float) * 2 * m), "memset") ||
                !rt(cudaMemset(s->vel, 0, sizeof(float) * 2 * m), "memset") ||
                !rt(cudaMemset(s->acc, 0, sizeof(float) * 2 * m), "memset") ||
                !rt(cudaMemset(s->dens, 0, sizeof(float) * m), "memset") ||
                !rt(cudaMemset(s->pres, 0, sizeof(float) * m), "memset") ||
                !rt(cudaMemset(s->vis, 0, sizeof(float) * m), "memset"))
                return false;
            unsigned um = static_cast<unsigned>(m);
            void* args[] = {&s->gl, &um};
            if (!launch(kInitIds, um, 0, args)) return false;
        }
        for (Grid* g : {&gL, &gH}) {
            const size_t m = static_cast<size_t>(g == &gL ? L.max : H.max);
            if (!alloc(&g->hash, m) || !alloc(&g->start, g->cells) || !alloc(&g->end, g->cells) ||
                !alloc(&g->ids[0], m) || !alloc(&g->ids[1], m))
                return false;
            unsigned um = static_cast<unsigned>(m);
            for (int k = 0; k < 2; ++k) {  // both id lists start as the identity (2358-2377)
                void* args[] = {&g->ids[k], &um};
                if (!launch(kInitIds, um, 0, args)) return false;
            }
        }
        if (!alloc(&stL, L.max) || !alloc(&stH, H.max) || !alloc(&trL[0], L.max) || !alloc(&trL[1], L.max) ||
            !alloc(&cntL, 1) || !alloc(&cntH, 1) || !alloc(&cntTrL, 1) || !alloc(&bHash, B.max) ||
            !alloc(&bIds, B.max) || !alloc(&bStart, gL.cells) || !alloc(&bEnd, gL.cells))
            return false;
        if (!rt(cudaMemset(stL, 0, L.max ? L.max : 1), "memset") || !rt(cudaMemset(stH, 0, H.max ? H.max : 1), "memset"))
            return false;
        if (n_low > 0) {
            if (!rt(cudaMemcpy(L.pos, low_pos, sizeof(float) * 2 * n_low, cudaMemcpyHostToDevice), "upload"))
                return false;
            if (low_vel && !rt(cudaMemcpy(L.vel, low_vel, sizeof(float) * 2 * n_low, cudaMemcpyHostToDevice), "upload"))
                return false;
        }
        if (n_wall > 0 &&
            !rt(cudaMemcpy(B.pos, wall_pos, sizeof(float) * 2 * n_wall, cudaMemcpyHostToDevice), "upload"))
            return false;
        if (!bind() || !init_boundaries()) return false;
        return rt(cudaDeviceSynchronize(), "create");
    }
};

}  // namespace

extern "C" {

// A reference solver on the GPU from the scene's arrays (tss_solver_create's
// arguments); NULL on failure with the reason in err.
void* refgpu_create(const char* cubin, const tss_config* cfg, int n_low, const float* low_pos, const float* low_vel,
                    float mass_low, int cap_high, float mass_high, int n_wall, const float* wall_pos,
                    float mass_wall, char* err, int err_len) {
    RefGpu* r = new RefGpu();
    if (!r->create(cubin, cfg, n_low, low_pos, low_vel, mass_low, cap_high, mass_high, n_wall, wall_pos,
                   mass_wall)) {
        if (err && err_len > 0) std::snprintf(err, static_cast<size_t>(err_len), "%s", r->err.c_str());
        delete r;
        return nullptr;
    }
    return r;
}

void refgpu_destroy(void* h) { delete static_cast<RefGpu*>(h); }

// n reference steps (each ends in the reference's synchronous count read-backs).
// 0 on success, else 1 with the reason in err.
int refgpu_step(void* h, int n, char* err, int err_len) {
    RefGpu* r = static_cast<RefGpu*>(h);
    for (int k = 0; k < n; ++k)
        if (!r->step()) {
            if (err && err_len > 0) std::snprintf(err, static_cast<size_t>(err_len), "%s", r->err.c_str());
            return 1;
        }
    return 0;
}

// Replaces the state (RefGpu::set_state).  0 on success, else 1 with the reason in err.
int refgpu_set_state(void* h, const float* low_pos, const float* low_vel, const unsigned char* low_state,
                     int n_high, const int* high_ids, const float* high_pos, const float* high_vel,
                     const unsigned char* high_state, char* err, int err_len) {
    RefGpu* r = static_cast<RefGpu*>(h);
    if (!r->set_state(low_pos, low_vel, low_state, n_high, high_ids, high_pos, high_vel, high_state)) {
        if (err && err_len > 0) std::snprintf(err, static_cast<size_t>(err_len), "%s", r->err.c_str());
        return 1;
    }
    return 0;
}

// {n_low, n_high, n_transient_low}
void refgpu_counts(void* h, int* out3) {
    RefGpu* r = static_cast<RefGpu*>(h);
    out3[0] = r->L.num;
    out3[1] = r->H.num;
    out3[2] = r->nTrL;
}

// Slot-indexed positions and velocities (2*cap floats each) and states (cap bytes)
// of a scale, read after synchronising.
int refgpu_state(void* h, int scale, float* pos, float* vel, unsigned char* state, int cap) {
    RefGpu* r = static_cast<RefGpu*>(h);
    const Sys& s = scale == 0 ? r->L : r->H;
    const int m = cap < s.max ? cap : s.max;
    if (m <= 0) return 0;
    if (cudaMemcpy(pos, s.pos, sizeof(float) * 2 * m, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
    if (cudaMemcpy(vel, s.vel, sizeof(float) * 2 * m, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
    if (cudaMemcpy(state, scale == 0 ? r->stL : r->stH, m, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
    return 0;
}

}  // extern "C"
