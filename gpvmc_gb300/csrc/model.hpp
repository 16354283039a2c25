// Host-side model of the sampling path: square lattice, magnetic-Brillouin-zone
// orbital enumeration, staggered-flux (+Neel) single-particle coefficients and
// the channel state sets.  Pure C++ on the host; the device consumes the
// tables it produces.
#pragma once

#include <complex>
#include <cstdint>
#include <vector>

namespace gv {

using zd = std::complex<double>;

// SquareLattice (SquareLattice.cpp:9-28): vertex v = y*L + x; edges created
// for x in [0,L), y in [0,L): first (v, v+y^), then (v, v+x^), each appended
// to both endpoints' edge lists.  nbr[v*4+e] is the e-th neighbour in that
// order, which is the order LatticeStepper::trystep draws from
// (LatticeStepper.cpp:45-47); edges[] keeps the creation order that ProjHeis
// iterates (ProjHeis.cpp:55-75).
struct Lattice {
    int L = 0, Ns = 0;
    std::vector<int32_t> nbr;       // Ns*4
    std::vector<int32_t> edge_i;    // 2*Ns
    std::vector<int32_t> edge_j;
};
Lattice make_square_lattice(int L);

// Orbital ("fock") index o in [0, Ns): o = 2*i + band, i the i-th magnetic
// Brillouin zone point in the enumeration order of StagFluxWaveFunction's
// constructor (StagFluxWaveFunction.cpp:24-41).
struct Orbitals {
    int L = 0, Ns = 0, Nk = 0;
    double bc[2] = {1.0, 1.0};
    std::vector<int32_t> kx, ky;     // Nk MBZ points (integer labels)
    std::vector<int32_t> qn2fock;    // (kx*L+ky)*2 + band -> orbital, Ns if not in MBZ
    bool ok = false;
};
Orbitals make_orbitals(int L, double bcx, double bcy);
bool in_mbz(const Orbitals& o, int kx, int ky);          // StagFluxWaveFunction.cpp:89-101
void mbz_fold(const Orbitals& o, int* k);                // StagFluxWaveFunction.cpp:103-119

// sqrt(2) * exp(i k.r) for MBZ point i and site s, stored [s*Nk + i]
// (StagFluxWaveFunction.cpp:55-63).
void phase_table(const Orbitals& o, std::vector<zd>& ph);

// U_k / V_k coefficients (StagFluxWaveFunction.cpp:121-163) for every orbital
// of flavour fl: coef[sub*Ns + o] = (sub == 0 ? U : V)(k_o, fl, band_o), so that
// phi_o(s) = phase[s][o/2] * coef[sublattice(s)][o] (sublattice = (x+y)%2).
// Returns false if a coefficient is NaN (delta_k = 0, matrix_element abort).
bool stagflux_coefs(const Orbitals& o, double phi, double neel, double neel_exp, int fl, zd* coef);

// phi_o(s) assembled exactly as StagFluxWaveFunction::matrix_element does.
zd phi_elem(const zd& phase, const zd& coef);

// Channel state set (StagFluxGroundState.cpp:3-15, StagFluxTransExciton.cpp:7-44).
// States are lists of occupied orbitals per flavour.  hops[(a*Nexc+b)*2+fl]
// is the one-orbital hop (from, to) of flavour fl going from state a to b,
// (-1,-1) if none (WaveFunction::AddState, WaveFunction.cpp:39-67).
struct Channel {
    int kind = 0;          // 0 groundstate, 1 transverse exciton, 2 longitudinal exciton
    int N[2] = {0, 0};
    int Nexc = 0;
    std::vector<int32_t> fock0[2];        // state 0 Fock vectors: orbital -> particle or N
    std::vector<int32_t> hop_from, hop_to; // (a*Nexc + b)*2 + fl
    // transverse exciton: flavour-0 upper-band orbital and flavour-1 hole of state k;
    // longitudinal exciton: the particle-hole pair (exc_up, exc_dn) of state k, in
    // flavour k % 2 for k < Ns, and -1 for the ground state (k = Ns)
    std::vector<int32_t> exc_up, exc_dn;
    bool ok = false;
};
Channel make_channel(const Orbitals& o, int kind, int qx, int qy);

}  // namespace gv
