// A small NpT run of the reference's Simulation with casino_gpu.patch applied, on the CPU path
// (no backend) or with rampack_gb300::GpuSimulationBackend attached, the way casino sets it up
// (src/frontend/modes/CasinoMode.cpp:171).
//
//   casino_gpu_check <cpu|gpu> <n> <spacing> <cycles> <adjust 0|1> <translation step> <box step>
//                    <pressure> <seed>
//
// n^3 hard spheres of radius 0.5 on a simple cubic lattice (positions (i + 0.5) * spacing) in a
// cubic box of side n * spacing; a TranslationSampler, a TriclinicDeltaScaler moving all
// entries, temperature 1; Simulation::integrate over `cycles` thermalisation cycles (adjust = 1)
// or averaging cycles (adjust = 0), one thread, no domain division.  Prints the final box (9
// values), then every position, as C99 hex floats, one value per line, then the translation and
// box-move counters.  Exit status 3 and a message on stderr when the backend fails (e.g. no
// CUDA device).
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "core/PeriodicBoundaryConditions.h"
#include "core/Simulation.h"
#include "core/move_samplers/TranslationSampler.h"
#include "core/shapes/SphereTraits.h"
#include "core/volume_scalers/TriclinicDeltaScaler.h"

#include "GpuSimulationBackend.hpp"

int main(int argc, char **argv) {
    if (argc != 10) {
        std::fprintf(stderr, "usage: %s <cpu|gpu> <n> <spacing> <cycles> <adjust> <tstep> <bstep> <pressure> <seed>\n",
                     argv[0]);
        return 2;
    }
    const std::string mode = argv[1];
    const int n = std::atoi(argv[2]);
    const double spacing = std::atof(argv[3]);
    const auto cycles = static_cast<std::size_t>(std::atoll(argv[4]));
    const bool adjust = std::atoi(argv[5]) != 0;
    const double tstep = std::atof(argv[6]);
    const double bstep = std::atof(argv[7]);
    const double pressure = std::atof(argv[8]);
    const auto seed = static_cast<unsigned long>(std::strtoull(argv[9], nullptr, 10));
    if (n <= 0 || cycles == 0 || (mode != "cpu" && mode != "gpu")) return 2;

    try {
        SphereTraits traits(0.5);
        std::vector<Shape> shapes;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++)
                    shapes.emplace_back(Vector<3>{(i + 0.5) * spacing, (j + 0.5) * spacing, (k + 0.5) * spacing});
        auto packing = std::make_unique<Packing>(TriclinicBox(n * spacing), std::move(shapes),
                                                 std::make_unique<PeriodicBoundaryConditions>(),
                                                 traits.getInteraction(), 1, 1);
        std::vector<std::unique_ptr<MoveSampler>> samplers;
        samplers.push_back(std::make_unique<TranslationSampler>(tstep));
        Simulation sim(std::move(packing), std::move(samplers), seed,
                       std::make_unique<TriclinicDeltaScaler>(bstep, true), {1, 1, 1}, false);
        if (mode == "gpu")
            sim.setBackend(std::make_shared<rampack_gb300::GpuSimulationBackend>(seed, std::array<bool, 3>{}));

        Simulation::Environment env;
        env.setTemperature(1.0);
        env.setPressure(pressure);
        Simulation::IntegrationParameters ip;
        if (adjust)
            ip.thermalisationCycles = cycles;
        else
            ip.averagingCycles = cycles;
        ip.averagingEvery = cycles;
        ip.snapshotEvery = cycles;
        ip.inlineInfoEvery = cycles;
        std::ostringstream sink;
        Logger logger(sink);
        sim.integrate(env, ip, traits, std::make_shared<ObservablesCollector>(), {}, logger);

        const Packing &fin = sim.getPacking();
        const auto &box = fin.getBox().getDimensions();
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) std::printf("%a\n", box(a, b));
        for (const auto &shape : fin)
            for (int d = 0; d < 3; d++) std::printf("%a\n", shape.getPosition()[d]);
        for (const auto &st : sim.getMovesStatistics())
            std::printf("# %s %zu %zu\n", st.groupName.c_str(), st.totalMoves, st.acceptedMoves);
    } catch (const std::exception &ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 3;
    }
    return 0;
}
