// dam_break_main.cpp -- the reference's main.cpp scene setup (TwoScale2D/main.cpp:
// 131-208) and frame loop (65-102) written against include/tss.hpp, headless.
// Built and run by tests/test_cpp_dropin.py; prints "n_low n_high steps".
#include <cmath>
#include <cstdio>
#include <memory>

#include "tss.hpp"

int main(int argc, char** argv) {
    const int frames = argc > 1 ? std::atoi(argv[1]) : 50;
    const float PI = 3.14159265358979323846f;
    try {
        // the reference's own dam break (main.cpp:144-154), 101 x 151 particles
        float restDensity = 1000.0f;
        float fluidVol = 100.0f * 0.0025f * 150.0f * 0.0025f;
        unsigned int numParticles = 101 * 151;
        float particleMass = fluidVol * restDensity / numParticles;
        float effectiveRadius = std::sqrt(fluidVol * 25.0f / (numParticles * PI));
        float effectiveRadiusHigh = 0.5f * effectiveRadius;
        float taitCoeff = 1119.0714f;
        float speedSound = 88.1472f;
        float alpha = 0.04f;
        float tensionCoefficient = 0.08f;
        float timeStep = 0.0002f;
        std::unique_ptr<tss::ParticleSystem> fluid(
            tss::CreateParticleBox(0.205f, 0.105f, 0.0025f, 101, 151, particleMass));
        tss::ParticleSystem fluidHigh(fluid->GetMaxParticles() * 4, fluid->GetMass() / 4.0f);
        std::unique_ptr<tss::ParticleSystem> walls(tss::CreateParticleBoxCanvas(
            0.1f, 0.1f, 0.0025f, 321, 321, 3, 3, 1000.0f * 0.25f * 0.25f / (101.0f * 151.0f)));
        tss::WCSPHConfig config(0.0f, 0.0f, 1.0f, 1.0f, effectiveRadius, effectiveRadiusHigh, restDensity,
                                taitCoeff, speedSound, alpha, tensionCoefficient, timeStep);
        tss::WCSPHSolver solver(config, *fluid, fluidHigh, *walls);
        solver.Bind();
        for (int i = 0; i < frames; ++i) solver.AdvanceTS();
        tss_counts c = solver.counts();
        std::printf("%d %d %lld\n", c.n_low, c.n_high, c.steps);
        if (c.error_bits) {
            std::printf("device error bits %u\n", c.error_bits);
            return 2;
        }
    } catch (const std::runtime_error& e) {
        std::printf("%s\n", e.what());
        return 1;
    }
    return 0;
}
