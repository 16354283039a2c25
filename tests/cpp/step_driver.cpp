// Step-level driver over the C++ adapter (include/gpvmc_gb300.hpp): one chain
// stepped the way MetroMC::Walk steps it (MetroMC.cpp:45-103) --
// LatticeStepper::trystep, MetroMC::YesNo on new_weight / state_weight,
// LatticeStepper::step on acceptance -- with every step printed, then the
// second half of the steps through MetroMC::Step itself.
//   step_driver gs|trans|long L phi_over_pi neel seed steps qx qy fp64|mixed
// Output lines:
//   S v1 v2 khop accepted ratio        one per step of the first half
//   V K Nr state <re im exp10 of VirtUpdate(rhop, khop, qs) for every state, no hop
//      and the first antiparallel bond> after the first half, with the current state
//   C <occupation of the sites>        final configuration (1 = flavour 0)
//   A re im exp10 state                final amplitude and channel state
#include <cstdio>
#include <cstdlib>
#include <string>

#include "gpvmc_gb300.hpp"

int main(int argc, char** argv)
{
    if (argc < 10) {
        std::fprintf(stderr, "usage: %s gs|trans|long L phi_over_pi neel seed steps qx qy fp64|mixed\n", argv[0]);
        return 2;
    }
    const std::string channel = argv[1];
    const int L = std::atoi(argv[2]);
    const double phi = std::atof(argv[3]) * M_PI;   // vmc.cpp:120
    const double neel = std::atof(argv[4]);
    const uint64_t seed = std::strtoull(argv[5], nullptr, 10);
    const int steps = std::atoi(argv[6]);
    const int qx = std::atoi(argv[7]), qy = std::atoi(argv[8]);
    const int prec = std::string(argv[9]) == "mixed" ? GV_PREC_MIXED : GV_PREC_FP64;
    try {
        gv::StagFluxGroundState gs(L, phi, neel);
        gv::StagFluxTransExciton tx(L, phi, neel, qx, qy);
        gv::StagFluxLongExciton lx(L, phi, neel, qx, qy);
        const gv::WaveFunctionParams& wav = channel == "trans"  ? static_cast<const gv::WaveFunctionParams&>(tx)
                                            : channel == "long" ? static_cast<const gv::WaveFunctionParams&>(lx)
                                                                : gs;
        gv::Job job(wav, 1, seed, prec);
        job.InitWalkers();
        gv::LatticeStepper stepper(job);
        gv::MetroMC varmc(stepper);
        // first half: MetroMC::Step written out, each step printed
        gv::BigDouble state_weight = stepper.weight();
        for (int s = 0; s < steps / 2; ++s) {
            const gv::BigDouble new_weight = stepper.trystep();
            const gv::BigDouble ratio = new_weight / state_weight;
            const int khop = stepper.Khop();   // the proposal's arg-max state, before step() clears it
            const bool acc = varmc.YesNo(ratio);
            if (acc) {
                stepper.step();
                state_weight = new_weight;
            }
            std::printf("S %d %d %d %d %.17e\n", stepper.Proposal(0), stepper.Proposal(1), khop, int(acc),
                        double(ratio));
        }
        // SlaterDeterminant::VirtUpdate with the reference's hop-path sets: the
        // empty real-space hop and the first antiparallel bond, against every
        // state of the wavefunction (LatticeStepper::weight / ProjHeis form)
        {
            const std::vector<int8_t> up = job.Config();
            std::vector<std::vector<gv::hop_path_t>> rhop(1, std::vector<gv::hop_path_t>(2));
            for (int y = 0; y < L && rhop.size() < 2; ++y)
                for (int x = 0; x < L && rhop.size() < 2; ++x) {
                    const int a = y * L + x, b = y * L + (x + 1) % L;
                    if (up[a] != up[b]) {
                        const int u = up[a] ? a : b, d = up[a] ? b : a;
                        std::vector<gv::hop_path_t> h(2);
                        h[0].push_back(gv::hop_t(u, d));
                        h[1].push_back(gv::hop_t(d, u));
                        rhop.push_back(h);
                    }
                }
            const auto khop = stepper.GetWaveFunction()->GetHops();
            std::vector<gv::BigComplex> qs;
            stepper.GetAmp()->VirtUpdate(rhop, khop, qs);
            std::printf("V %d %d %d", int(khop.size()), int(rhop.size()), stepper.GetWaveFunction()->GetCurrentState());
            for (const auto& q : qs) std::printf(" %.17e %.17e %d", q.mantissa().real(), q.mantissa().imag(), q.exponent10());
            std::printf("\n");
        }
        // second half: MetroMC::Step itself
        for (int s = steps / 2; s < steps; ++s) varmc.Step(false);
        const std::vector<int8_t> up = job.Config();
        std::printf("C");
        for (int8_t u : up) std::printf(" %d", int(u));
        const gv::BigComplex a = stepper.GetAmp()->Amp();
        std::printf("\nA %.17e %.17e %d %d\n", a.mantissa().real(), a.mantissa().imag(), a.exponent10(),
                    stepper.GetWaveFunction()->GetCurrentState());
    } catch (const gv::Error& err) {
        std::fprintf(stderr, "error: %s\n", err.what());
        return 1;
    }
    return 0;
}
