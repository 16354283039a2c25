// A vmc.cpp-style driver (vmc.cpp:140-318) written against the C++ adapter
// include/gpvmc_gb300.hpp: the reference's object names, one job of W chains.
//   vmc_driver L phi_over_pi neel seed walkers therm_sweeps meas_sweeps precision
// Prints one line: per-walker E/site (ProjHeis), staggered magnetisation and
// the rejection ratio of walker 0.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "gpvmc_gb300.hpp"

int main(int argc, char** argv)
{
    if (argc < 9) {
        std::fprintf(stderr, "usage: %s L phi_over_pi neel seed walkers therm_sweeps meas_sweeps fp64|mixed\n", argv[0]);
        return 2;
    }
    const int L = std::atoi(argv[1]);
    const double phi = std::atof(argv[2]) * M_PI;   // vmc.cpp:120
    const double neel = std::atof(argv[3]);
    const uint64_t seed = std::strtoull(argv[4], nullptr, 10);
    const int walkers = std::atoi(argv[5]);
    const int therm = std::atoi(argv[6]);
    const int sweeps = std::atoi(argv[7]);
    const int prec = std::string(argv[8]) == "mixed" ? GV_PREC_MIXED : GV_PREC_FP64;
    try {
        gv::StagFluxGroundState wav(L, phi, neel);
        gv::Job job(wav, walkers, seed, prec);
        gv::SlaterDeterminant amp(job);
        gv::LatticeStepper step(job);
        gv::MetroMC varmc(step);
        gv::ProjHeis heis(step);
        gv::StagMagnZ stag(step);
        varmc.AddQuantity(&heis);
        varmc.AddQuantity(&stag);
        job.InitWalkers();
        varmc.Walk(uint64_t(therm) * L * L, 0);
        varmc.Walk(uint64_t(sweeps) * L * L, uint64_t(L) * L);
        const auto e = heis.save();
        const auto m = stag.save();
        std::printf("E");
        for (const auto& x : e) std::printf(" %.15e", x.real());
        std::printf(" M");
        for (const auto& x : m) std::printf(" %.15e", x.real());
        std::printf(" R %.15e N %d\n", varmc.Rejection(0), heis.GetNmeas(0));
    } catch (const gv::Error& err) {
        std::fprintf(stderr, "error: %s\n", err.what());
        return 1;
    }
    return 0;
}
