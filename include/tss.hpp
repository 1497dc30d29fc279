// tss.hpp -- header-only C++ drop-in for the reference's solver classes, over the C
// ABI of tss.h.  Same class names, constructor arguments, method names and error
// behaviour (std::runtime_error) as TwoScale2D/WCSPHSolver.h:14-131 and
// TwoScale2D/ParticleSystem.h:17-86, so the reference's main.cpp (init(),
// display()) compiles against it with the GL/renderer lines removed:
//
//   tss::WCSPHConfig config(0, 0, 1, 1, r, r/2, rho0, B, c, alpha, sigma, dt);
//   tss::ParticleSystem* fluid = tss::CreateParticleBox(xs, ys, dx, nx, ny, m);
//   tss::ParticleSystem high(fluid->GetMaxParticles() * 4, fluid->GetMass() / 4);
//   tss::ParticleSystem* walls = tss::CreateParticleBoxCanvas(...);
//   tss::WCSPHSolver solver(config, *fluid, high, *walls);
//   solver.Bind();
//   for (;;) solver.AdvanceTS();          // per frame
//
// Differences: a ParticleSystem collects particles on the host until a solver
// binds it; afterwards Positions()/Densities()/ParticleIDs() return DEVICE
// pointers into the solver's buffers (the reference returned mapped GL buffers)
// and GetNumParticles() reads the device count.  Map()/Unmap() are no-ops.
#ifndef TSS_HPP
#define TSS_HPP

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "tss.h"

namespace tss {

inline void throw_on(tss_status st, tss_solver* s = nullptr) {
    if (st == TSS_OK) return;
    std::string msg = tss_status_string(st);
    if (s) {
        char buf[512];
        if (tss_solver_last_error(s, buf, sizeof buf) == TSS_OK && buf[0]) msg += std::string(": ") + buf;
    }
    throw std::runtime_error(msg);
}

// WCSPHConfig (WCSPHSolver.h:14-35); throws on xs >= xe || ys >= ye like the
// reference constructor (WCSPHSolver.cu:2312-2316).
struct WCSPHConfig {
    WCSPHConfig(float xs, float ys, float xe, float ye, float effectiveRadius, float effectiveRadiusHigh,
                float restDensity, float taitCoeff, float speedSound, float alpha, float tensionCoefficient,
                float timeStep) {
        if (tss_config_init(&cfg, xs, ys, xe, ye, effectiveRadius, effectiveRadiusHigh, restDensity, taitCoeff,
                            speedSound, alpha, tensionCoefficient, timeStep) != TSS_OK)
            throw std::runtime_error("Invalid configuration parameters");
        DomainOrigin[0] = cfg.domain_origin[0];
        DomainOrigin[1] = cfg.domain_origin[1];
        DomainEnd[0] = cfg.domain_end[0];
        DomainEnd[1] = cfg.domain_end[1];
        DomainDimensions[0] = cfg.dims_low[0];
        DomainDimensions[1] = cfg.dims_low[1];
        DomainDimensionsHigh[0] = cfg.dims_high[0];
        DomainDimensionsHigh[1] = cfg.dims_high[1];
        EffectiveRadius = effectiveRadius;
        EffectiveRadiusHigh = effectiveRadiusHigh;
        RestDensity = restDensity;
        TaitCoeffitient = taitCoeff;
        SpeedSound = speedSound;
        Alpha = alpha;
        TensionCoefficient = tensionCoefficient;
        TimeStep = timeStep;
    }
    float DomainOrigin[2];
    float DomainEnd[2];
    int DomainDimensions[2];
    int DomainDimensionsHigh[2];
    float EffectiveRadius, EffectiveRadiusHigh, RestDensity, TaitCoeffitient, SpeedSound, Alpha,
        TensionCoefficient, TimeStep;
    tss_config cfg;  // the full configuration (ROI, relaxation, flags) for tuning
};

class WCSPHSolver;

// ParticleSystem (ParticleSystem.h:17-78).
class ParticleSystem {
public:
    ParticleSystem(unsigned int maxParticles, float mass) : mMax(maxParticles), mMass(mass) {}
    ParticleSystem(const ParticleSystem&) = delete;
    ParticleSystem& operator=(const ParticleSystem&) = delete;

    void PushParticle(float position[2]) {
        if (mSolver) throw std::runtime_error("Positions is not mapped");
        if (mPos.size() / 2 >= mMax) throw std::runtime_error("particle system is full");
        mPos.push_back(position[0]);
        mPos.push_back(position[1]);
    }
    void Map() {}
    void Unmap() {}
    inline float* Positions();
    inline float* Velocities();
    inline float* Densities();
    inline int* ParticleIDs();
    float GetMass() const { return mMass; }
    inline unsigned int GetNumParticles() const;
    unsigned int GetMaxParticles() const { return mMax; }

private:
    friend class WCSPHSolver;
    unsigned int mMax;
    float mMass;
    std::vector<float> mPos;  // host staging until bound
    WCSPHSolver* mSolver = nullptr;
    int mScale = TSS_SCALE_LOW;
};

// WCSPHSolver (WCSPHSolver.h:37-131).
class WCSPHSolver {
public:
    WCSPHSolver(const WCSPHConfig& config, ParticleSystem& fluidParticles, ParticleSystem& fluidParticlesHigh,
                ParticleSystem& boundaryParticles)
        : mCfg(config.cfg), mLow(fluidParticles), mHigh(fluidParticlesHigh), mWalls(boundaryParticles) {}
    ~WCSPHSolver() {
        if (mS) tss_solver_destroy(mS);
    }
    WCSPHSolver(const WCSPHSolver&) = delete;
    WCSPHSolver& operator=(const WCSPHSolver&) = delete;

    // Upload everything and build the boundary grid (WCSPHSolver::Bind, 2537-2639).
    void Bind() {
        if (mS) return;
        const int nL = static_cast<int>(mLow.mPos.size() / 2);
        const int nW = static_cast<int>(mWalls.mPos.size() / 2);
        throw_on(tss_solver_create(&mCfg, nL, mLow.mPos.data(), nullptr, mLow.GetMass(),
                                   static_cast<int>(mHigh.GetMaxParticles()), mHigh.GetMass(), nW,
                                   mWalls.mPos.data(), mWalls.GetMass(), &mS));
        mLow.mSolver = this;
        mLow.mScale = TSS_SCALE_LOW;
        mHigh.mSolver = this;
        mHigh.mScale = TSS_SCALE_HIGH;
    }
    void Unbind() {}
    void Advance() {}      // empty in the reference (2649-2685)
    void AdvanceHigh() {}  // empty in the reference (2687-2724)
    // One two-scale step (AdvanceTS, 2726-2810), enqueued on the solver's stream.
    void AdvanceTS() {
        if (!mS) Bind();
        throw_on(tss_solver_step(mS, 1, nullptr), mS);
    }
    tss_solver* handle() { return mS; }

    // The gathers' arithmetic (tss_solver_set_arith; not in the reference): false
    // (the default) keeps the reference's FP32 arithmetic bit for bit, true spends
    // the step's 1e-5 tolerance on approximate square roots and reciprocals.
    void SetFastArithmetic(bool on) {
        if (!mS) Bind();
        throw_on(tss_solver_set_arith(mS, on ? TSS_ARITH_FAST : TSS_ARITH_EXACT), mS);
    }

    // Launch-shape autotuner (tss_solver_autotune; not in the reference): times the
    // candidate shapes on this solver's own steps, which advance its state, and
    // installs the fastest per gather.
    tss_launch Autotune(int stepsPerTrial = 3) {
        if (!mS) Bind();
        tss_launch l;
        throw_on(tss_solver_autotune(mS, stepsPerTrial, &l, nullptr), mS);
        return l;
    }

    tss_buffers buffers() {
        tss_buffers b;
        throw_on(tss_solver_device_buffers(mS, &b), mS);
        return b;
    }
    tss_counts counts() {
        tss_counts c;
        throw_on(tss_solver_counts(mS, &c), mS);
        return c;
    }

private:
    tss_config mCfg;
    ParticleSystem& mLow;
    ParticleSystem& mHigh;
    ParticleSystem& mWalls;
    tss_solver* mS = nullptr;
};

inline float* ParticleSystem::Positions() {
    if (!mSolver) return mPos.data();
    return const_cast<float*>(mSolver->buffers().pos[mScale]);
}
inline float* ParticleSystem::Velocities() {
    return mSolver ? const_cast<float*>(mSolver->buffers().vel[mScale]) : nullptr;
}
inline float* ParticleSystem::Densities() {
    return mSolver ? const_cast<float*>(mSolver->buffers().dens[mScale]) : nullptr;
}
inline int* ParticleSystem::ParticleIDs() {
    return mSolver ? const_cast<int*>(mSolver->buffers().id[mScale]) : nullptr;
}
inline unsigned int ParticleSystem::GetNumParticles() const {
    if (!mSolver) return static_cast<unsigned int>(mPos.size() / 2);
    tss_counts c = mSolver->counts();
    return static_cast<unsigned int>(mScale == TSS_SCALE_LOW ? c.n_low : c.n_high);
}

// CreateParticleBox (ParticleSystem.cpp:123-148): row-major lattice, j outer.
inline ParticleSystem* CreateParticleBox(float xs, float ys, float dx, unsigned int dimX, unsigned int dimY,
                                         float particleMass) {
    ParticleSystem* ps = new ParticleSystem(dimX * dimY, particleMass);
    for (unsigned int j = 0; j < dimY; j++)
        for (unsigned int i = 0; i < dimX; i++) {
            float pos[2] = {xs + dx * i, ys + dx * j};
            ps->PushParticle(pos);
        }
    return ps;
}

// CreateParticleBoxCanvas (ParticleSystem.cpp:150-179): the wall ring.
inline ParticleSystem* CreateParticleBoxCanvas(float xs, float ys, float dx, int dimX, int dimY, int offX, int offY,
                                               float particleMass) {
    unsigned int n = (dimX + 2 * offX) * (dimY + 2 * offY) - dimX * dimY;
    ParticleSystem* ps = new ParticleSystem(n, particleMass);
    for (int j = -offY; j < dimY + offY; j++)
        for (int i = -offX; i < dimX + offX; i++)
            if (i < 0 || i >= dimX || j < 0 || j >= dimY) {
                float pos[2] = {xs + dx * i, ys + dx * j};
                ps->PushParticle(pos);
            }
    return ps;
}

}  // namespace tss

#endif  // TSS_HPP
