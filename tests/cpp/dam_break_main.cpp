// dam_break_main.cpp -- the reference's main.cpp scene setup (TwoScale2D/main.cpp:
// 131-208) and frame loop (65-102) written against include/tss.hpp, headless.
// Built and run by tests/test_cpp_dropin.py; prints "n_low n_high steps" and, given
// a second argument, writes the scene's constants and the final state of both
// scales (tss_solver_download) to that file for a comparison with the oracle.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <vector>

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
        if (argc > 2) {  // constants, then per scale: n, ids, pos, vel, state, dens
            FILE* f = std::fopen(argv[2], "wb");
            if (!f) throw std::runtime_error("cannot write the state file");
            const float consts[9] = {particleMass, effectiveRadius, effectiveRadiusHigh, taitCoeff, speedSound,
                                     alpha, tensionCoefficient, timeStep, walls->GetMass()};
            std::fwrite(consts, sizeof(float), 9, f);
            for (int scale = 0; scale < 2; ++scale) {
                const int n = scale == 0 ? c.n_low : c.n_high;
                std::vector<int32_t> id(n);
                std::vector<float> pos(2 * n), vel(2 * n), dens(n);
                std::vector<uint8_t> st(n);
                tss_scale_state out{n, id.data(), pos.data(), vel.data(), st.data(), dens.data(), nullptr};
                if (tss_solver_download(solver.handle(), scale, &out) != TSS_OK)
                    throw std::runtime_error("download failed");
                std::fwrite(&n, sizeof(int), 1, f);
                std::fwrite(id.data(), sizeof(int32_t), n, f);
                std::fwrite(pos.data(), sizeof(float), 2 * n, f);
                std::fwrite(vel.data(), sizeof(float), 2 * n, f);
                std::fwrite(st.data(), 1, n, f);
                std::fwrite(dens.data(), sizeof(float), n, f);
            }
            std::fclose(f);
        }
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
