// Host-side model tables for the sampling path (see model.hpp).  Compiled
// with -ffp-contract=off so that the staggered-flux tables are the same
// IEEE doubles on x86_64 and aarch64 hosts.
#include "model.hpp"

#include <cmath>

namespace gv {

Lattice make_square_lattice(int L)
{
    Lattice lat;
    lat.L = L;
    lat.Ns = L * L;
    lat.nbr.assign(size_t(lat.Ns) * 4, -1);
    std::vector<int> deg(lat.Ns, 0);
    for (int x = 0; x < L; ++x)
        for (int y = 0; y < L; ++y) {
            int a = y * L + x;
            int ends[2] = {((y + 1) % L) * L + x, y * L + (x + 1) % L};
            for (int b : ends) {
                lat.edge_i.push_back(a);
                lat.edge_j.push_back(b);
                if (deg[a] < 4) lat.nbr[a * 4 + deg[a]] = b;
                ++deg[a];
                if (deg[b] < 4) lat.nbr[b * 4 + deg[b]] = a;
                ++deg[b];
            }
        }
    return lat;
}

bool in_mbz(const Orbitals& o, int kx, int ky)
{
    double kkx = (double(kx) + o.bc[0] / 2.0) / double(o.L);
    double kky = (double(ky) + o.bc[1] / 2.0) / double(o.L);
    double eps = 1e-9;
    return (kkx >= 0 && kkx < 1 && kky >= 0 && kky < 1) &&
           (kkx + kky - 0.5 < 0 || kkx + kky - 1.5 >= -eps || kky - kkx - 0.5 > eps ||
            kky - kkx + 0.5 <= eps);
}

void mbz_fold(const Orbitals& o, int* k)
{
    int h = o.L / 2;
    if (in_mbz(o, k[0], k[1])) return;
    k[0] += (k[0] < h) ? h : -h;
    k[1] += (k[1] < h) ? h : -h;
}

Orbitals make_orbitals(int L, double bcx, double bcy)
{
    Orbitals o;
    o.L = L;
    o.Ns = L * L;
    o.bc[0] = bcx;
    o.bc[1] = bcy;
    o.qn2fock.assign(size_t(2) * o.Ns, o.Ns);
    for (int kx = 0; kx < L; ++kx)
        for (int ky = 0; ky < L; ++ky)
            if (in_mbz(o, kx, ky)) {
                int i = int(o.kx.size());
                o.kx.push_back(kx);
                o.ky.push_back(ky);
                if (2 * i + 1 < 2 * o.Ns) {
                    o.qn2fock[(kx * L + ky) * 2] = 2 * i;
                    o.qn2fock[(kx * L + ky) * 2 + 1] = 2 * i + 1;
                }
            }
    o.Nk = int(o.kx.size());
    o.ok = (2 * o.Nk == o.Ns);
    return o;
}

static void kvec(const Orbitals& o, int i, double* k)
{
    k[0] = (double(o.kx[i]) + o.bc[0] / (2.0)) * 2 * M_PI / double(o.L);
    k[1] = (double(o.ky[i]) + o.bc[1] / (2.0)) * 2 * M_PI / double(o.L);
}

void phase_table(const Orbitals& o, std::vector<zd>& ph)
{
    const zd I(0, 1);
    ph.assign(size_t(o.Ns) * o.Nk, zd(0, 0));
    for (int s = 0; s < o.Ns; ++s) {
        double r[2];
        r[1] = double(s / o.L);
        r[0] = double(s) - r[1] * double(o.L);
        for (int i = 0; i < o.Nk; ++i) {
            double k[2];
            kvec(o, i, k);
            ph[size_t(s) * o.Nk + i] = std::sqrt(2.0) * std::exp(I * (k[0] * r[0] + k[1] * r[1]));
        }
    }
}

namespace {
struct SF {
    double phi, neel, ne;
    zd delta(const double* k) const
    {
        return 0.5 * (std::cos(k[0]) * std::polar(1.0, phi) + std::cos(k[1]) * std::polar(1.0, -phi));
    }
    double neelk(const double* k) const
    {
        if (ne == 0.0) return neel;
        return neel * std::pow(0.5 * (std::pow(std::cos(k[0]), 2) + std::pow(std::cos(k[1]), 2)), ne);
    }
    double omega(const double* k) const { return std::sqrt(std::pow(neelk(k), 2) + std::norm(delta(k))); }
    zd U(const double* k, bool up, int band) const
    {
        double om = omega(k);
        zd d = delta(k);
        double nk = neelk(k);
        int sig = 2 * int(!up) - 1;
        if (band == 0) return std::sqrt(0.5 * zd(1 + sig * nk / om));
        return -std::conj(d) / std::abs(d) * std::sqrt(0.5 * zd(1 - sig * nk / om));
    }
    zd V(const double* k, bool up, int band) const
    {
        double om = omega(k);
        zd d = delta(k);
        double nk = neelk(k);
        int sig = 2 * int(!up) - 1;
        if (band == 0) return d / std::abs(d) * std::sqrt(0.5 * zd(1 - sig * nk / om));
        return std::sqrt(0.5 * zd(1 + sig * nk / om));
    }
};
}  // namespace

bool stagflux_coefs(const Orbitals& o, double phi, double neel, double neel_exp, int fl, zd* coef)
{
    SF sf{phi, neel, neel_exp};
    bool up = fl != 0;   // matrix_element(f, r, s) passes the flavour index as `up`
    bool ok = true;
    for (int orb = 0; orb < o.Ns; ++orb) {
        double k[2];
        kvec(o, orb / 2, k);
        int band = orb % 2;
        zd u = sf.U(k, up, band), v = sf.V(k, up, band);
        for (int sub = 0; sub < 2; ++sub) {
            zd c = double(1 - sub) * u + double(sub) * v;
            if (std::isnan(c.real()) || std::isnan(c.imag())) ok = false;
            coef[size_t(sub) * o.Ns + orb] = c;
        }
    }
    return ok;
}

zd phi_elem(const zd& ph, const zd& c)
{
    double a = ph.real(), b = ph.imag(), x = c.real(), y = c.imag();
    return zd(a * x - b * y, a * y + b * x);
}

Channel make_channel(const Orbitals& o, int kind, int qx, int qy)
{
    Channel ch;
    ch.kind = kind;
    int Ns = o.Ns, L = o.L;
    std::vector<std::vector<char>> occ[2];   // per flavour: per state occupancy over orbitals
    if (kind == 0) {
        ch.N[0] = ch.N[1] = Ns / 2;
        std::vector<char> s(Ns, 0);
        for (int f = 0; f < Ns / 2; ++f) s[2 * f] = 1;
        occ[0].push_back(s);
        occ[1].push_back(s);
    } else if (kind == 1) {
        ch.N[0] = Ns / 2 + 1;
        ch.N[1] = Ns / 2 - 1;
        for (int fe = 0; fe < Ns / 2; ++fe) {
            int Qk[2] = {((o.kx[fe] - qx) % L + L) % L, ((o.ky[fe] - qy) % L + L) % L};
            mbz_fold(o, Qk);
            int hole = o.qn2fock[(Qk[0] * L + Qk[1]) * 2];
            std::vector<char> su(Ns, 0), sd(Ns, 0);
            for (int f = 0; f < Ns / 2; ++f) {
                su[2 * f] = 1;
                if (hole != 2 * f) sd[2 * f] = 1;
            }
            su[2 * fe + 1] = 1;
            occ[0].push_back(su);
            occ[1].push_back(sd);
            ch.exc_up.push_back(2 * fe + 1);
            ch.exc_dn.push_back(hole);
        }
    } else if (kind == 2) {
        // StagFluxLongExciton.cpp:6-66: for every upper-band orbital 2fe+1 the
        // particle-hole pair (2fe+1, hole of k - q) in flavour 0 (state 2fe) or
        // in flavour 1 (state 2fe+1); at q = 0 or (pi, pi) also the ground
        // state (state Ns).  The states differ by up to two orbital hops in one
        // flavour, so the single-hop table below is not built for this channel.
        ch.N[0] = ch.N[1] = Ns / 2;
        for (int fe = 0; fe < Ns / 2; ++fe) {
            int Qk[2] = {((o.kx[fe] - qx) % L + L) % L, ((o.ky[fe] - qy) % L + L) % L};
            mbz_fold(o, Qk);
            const int hole = o.qn2fock[(Qk[0] * L + Qk[1]) * 2];
            std::vector<char> full(Ns, 0), holed(Ns, 0);
            for (int f = 0; f < Ns / 2; ++f) {
                full[2 * f] = 1;
                if (hole != 2 * f) holed[2 * f] = 1;
            }
            holed[2 * fe + 1] = 1;
            for (int which = 0; which < 2; ++which) {
                occ[0].push_back(which == 0 ? holed : full);
                occ[1].push_back(which == 0 ? full : holed);
                ch.exc_up.push_back(2 * fe + 1);
                ch.exc_dn.push_back(hole);
            }
        }
        if ((qx == 0 && qy == 0) || (qx == L / 2 && qy == L / 2)) {
            std::vector<char> full(Ns, 0);
            for (int f = 0; f < Ns / 2; ++f) full[2 * f] = 1;
            occ[0].push_back(full);
            occ[1].push_back(full);
            ch.exc_up.push_back(-1);
            ch.exc_dn.push_back(-1);
        }
        ch.Nexc = int(occ[0].size());
        for (int fl = 0; fl < 2; ++fl) {
            ch.fock0[fl].assign(Ns, ch.N[fl]);
            int p = 0;
            for (int x = 0; x < Ns; ++x)
                if (occ[fl][0][x]) ch.fock0[fl][x] = p++;
            if (p != ch.N[fl]) return ch;
        }
        ch.ok = true;
        return ch;
    } else {
        return ch;
    }
    ch.Nexc = int(occ[0].size());
    for (int fl = 0; fl < 2; ++fl) {
        ch.fock0[fl].assign(Ns, ch.N[fl]);
        int p = 0;
        for (int x = 0; x < Ns; ++x)
            if (occ[fl][0][x]) ch.fock0[fl][x] = p++;
        if (p != ch.N[fl]) return ch;
    }
    size_t n = size_t(ch.Nexc) * ch.Nexc * 2;
    ch.hop_from.assign(n, -1);
    ch.hop_to.assign(n, -1);
    for (int a = 0; a < ch.Nexc; ++a)
        for (int b = 0; b < ch.Nexc; ++b)
            for (int fl = 0; fl < 2; ++fl) {
                int from = -1, to = -1, nf = 0, nt = 0;
                for (int x = 0; x < Ns; ++x) {
                    if (occ[fl][a][x] && !occ[fl][b][x]) { from = x; ++nf; }
                    if (!occ[fl][a][x] && occ[fl][b][x]) { to = x; ++nt; }
                }
                if (nf > 1 || nt > 1 || nf != nt) return ch;
                ch.hop_from[(size_t(a) * ch.Nexc + b) * 2 + fl] = from;
                ch.hop_to[(size_t(a) * ch.Nexc + b) * 2 + fl] = to;
            }
    ch.ok = true;
    return ch;
}

}  // namespace gv
