/*
 * vmc_oracle.c -- CPU restatement of the gpvmc Metropolis sampling path.
 *
 * TEST INFRASTRUCTURE ONLY (see vmc_oracle.h): the parity oracle and the
 * timed CPU baseline.  Never linked or loaded by the product.
 *
 * The code restates, in C, the algorithm of the reference files cited beside
 * each function: the same object state (State/WaveFunction/LatticeState),
 * the same extended-range arithmetic (BigComplex/BigDouble, base-10
 * mantissa/exponent), the same determinant-lemma and Woodbury formulas
 * (linalg::DetUpdate/InvUpdate) including the full A^-1*C matrix-vector
 * product of the reference's column-update branch, so that its cost per step
 * is representative of the reference CPU path.  BLAS/LAPACK calls of the
 * reference are written out as plain loops (column-major, LAPACK pivoting
 * rule |re|+|im|).  Only single-hop-per-flavour hop sets occur on this path
 * (nearest-neighbour spin exchanges, one-orbital exciton hops); larger ranks
 * are rejected with ORC_ERR_INVALID.
 */
#include "vmc_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex zc;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static _Thread_local int tl_err = 0;
static zc cplx(double re, double im);
static void set_err(int e) { if (!tl_err) tl_err = e; }

/* ------------------------------------------------------------------ */
/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11.  Multipliers and Weyl key increments as
 * published in that paper. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* 52 random bits -> double in (0,1), exactly: (m + 1/2) * 2^-52. */
double orc_u01(uint32_t a, uint32_t b)
{
    uint64_t m = ((uint64_t)a << 20) ^ (uint64_t)(b >> 12);
    m &= ((uint64_t)1 << 52) - 1;
    return ((double)m + 0.5) * 0x1p-52;
}

/* Counter layout: {call_lo, call_hi, walker, stream}, key {seed_lo, seed_hi};
 * each call yields two uniforms (words 0,1 then words 2,3). */
double orc_uniform_at(uint64_t seed, uint32_t walker, uint32_t stream, uint64_t k)
{
    uint64_t call = k >> 1;
    uint32_t ctr[4] = {(uint32_t)call, (uint32_t)(call >> 32), walker, stream};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t x[4];
    orc_philox4x32_10(ctr, key, x);
    return (k & 1) ? orc_u01(x[2], x[3]) : orc_u01(x[0], x[1]);
}

typedef struct {
    uint64_t seed;
    uint32_t walker, stream;
    uint64_t next;      /* index of the next uniform */
} rng_t;

static double rng_uniform(rng_t* r)
{
    return orc_uniform_at(r->seed, r->walker, r->stream, r->next++);
}

/* ------------------------------------------------------------------ */
/* BigComplex / BigDouble (BigComplex.h:10-367, BigDouble.h:11-353):
 * mantissa with |m| in [1,10) (or 0) and a base-10 exponent, renormalised by
 * repeated division/multiplication by 10 after every operation. */
typedef struct { zc c; int e; } bigc;
typedef struct { double c; int e; } bigd;

static void bigc_bound(bigc* x)   /* BigComplex.h:16-44 */
{
    double re = creal(x->c), im = cimag(x->c);
    if (isnan(re) || isinf(re) || isnan(im) || isinf(im)) { set_err(ORC_ERR_NAN); return; }
    while (cabs(x->c) > 10.0) { x->c /= 10.0; x->e++; }
    if (cabs(x->c) > 0) {
        while (cabs(x->c) < 1.0) { x->c *= 10.0; x->e--; }
    }
}

static void bigd_bound(bigd* x)   /* BigDouble.h:17-50 */
{
    if (isnan(x->c)) { set_err(ORC_ERR_NAN); return; }
    if (isinf(x->c)) return;
    while (fabs(x->c) > 10.0) { x->c /= 10.0; x->e++; }
    if (fabs(x->c) > 0) {
        while (fabs(x->c) < 1.0) { x->c *= 10.0; x->e--; }
    } else x->e = 0;
}

static bigc bigc_make(zc c, int e) { bigc r = {c, e}; bigc_bound(&r); return r; }
static bigd bigd_make(double c, int e) { bigd r = {c, e}; bigd_bound(&r); return r; }
static bigc bigc_mul(bigc a, bigc b) { return bigc_make(a.c * b.c, a.e + b.e); }
static bigc bigc_mul_d(bigc a, double d) { return bigc_make(a.c * d, a.e); }
static bigc bigc_div_d(bigc a, double d) { return bigc_make(a.c / d, a.e); }
static bigc bigc_div_bd(bigc a, bigd b) { return bigc_make(a.c / b.c, a.e - b.e); }
static bigc bigc_conj(bigc a) { return bigc_make(conj(a.c), a.e); }
static bigc bigc_add(bigc a, bigc b)
{
    int m = a.e > b.e ? a.e : b.e;
    return bigc_make(a.c * pow(10.0, a.e - m) + b.c * pow(10.0, b.e - m), m);
}
static void bigc_addeq(bigc* a, bigc b)
{
    int m = a->e > b.e ? a->e : b.e;
    a->c = a->c * pow(10.0, a->e - m) + b.c * pow(10.0, b.e - m);
    a->e = m;
    bigc_bound(a);
}
static void bigc_subeq(bigc* a, bigc b)
{
    int m = a->e > b.e ? a->e : b.e;
    a->c = a->c * pow(10.0, a->e - m) - b.c * pow(10.0, b.e - m);
    a->e = m;
    bigc_bound(a);
}
static void bigc_muleq(bigc* a, bigc b) { a->c *= b.c; a->e += b.e; bigc_bound(a); }
static zc bigc_z(bigc a) { return a.c * pow(10.0, a.e); }
static bigd bigc_norm(bigc a)     /* BigComplex.h:237-240 */
{
    double n = creal(a.c) * creal(a.c) + cimag(a.c) * cimag(a.c);
    return bigd_make(n, 2 * a.e);
}
static double bigd_d(bigd a) { return a.c * pow(10.0, a.e); }
static void bigd_addeq(bigd* a, bigd b)
{
    int m = a->e > b.e ? a->e : b.e;
    a->c = a->c * pow(10.0, a->e - m) + b.c * pow(10.0, b.e - m);
    a->e = m;
    bigd_bound(a);
}
static bigd bigd_div(bigd a, bigd b) { return bigd_make(a.c / b.c, a.e - b.e); }
static int bigd_lt(bigd l, bigd r)   /* BigDouble.h operator< */
{
    bigd_bound(&l); bigd_bound(&r);
    return l.e < r.e || (l.e == r.e && l.c < r.c);
}
static int bigd_gt(bigd l, bigd r)
{
    bigd_bound(&l); bigd_bound(&r);
    return l.e > r.e || (l.e == r.e && l.c > r.c);
}
static int bigc_is_zero(bigc a) { zc z = bigc_z(a); return creal(z) == 0.0 && cimag(z) == 0.0; }

/* ------------------------------------------------------------------ */
/* Hop sets: at most one hop per flavour (2 flavours). */
/* hop_path_t per flavour (defs.h:5-7): up to two hops (a long-exciton state
 * differs from another by two orbital hops in one flavour); hop 0 in
 * from/to, hop 1 in from2/to2. */
typedef struct { int n[2]; int from[2]; int to[2]; int from2[2]; int to2[2]; } hopset;

static hopset hopset_empty(void) { hopset h; memset(&h, 0, sizeof h); return h; }
static int hop_from(const hopset* h, int fl, int i) { return i ? h->from2[fl] : h->from[fl]; }
static int hop_to(const hopset* h, int fl, int i) { return i ? h->to2[fl] : h->to[fl]; }

/* State (State.cpp): m_fock[fl][s] = particle or Npt, m_part[fl][p] = s. */
typedef struct {
    int Nfl;
    int Npt[2], Nfs[2];
    int* fock[2];
    int* part[2];
    int sign;
} state_t;

static void state_init(state_t* s, const int Npt[2], const int Nfs[2])   /* State.cpp:204-217 */
{
    s->Nfl = 2;
    s->sign = 1;
    for (int fl = 0; fl < 2; ++fl) {
        s->Npt[fl] = Npt[fl];
        s->Nfs[fl] = Nfs[fl];
        s->fock[fl] = (int*)malloc(sizeof(int) * Nfs[fl]);
        s->part[fl] = (int*)malloc(sizeof(int) * (Npt[fl] > 0 ? Npt[fl] : 1));
        for (int i = 0; i < Nfs[fl]; ++i) s->fock[fl][i] = Npt[fl];
        for (int i = 0; i < Npt[fl]; ++i) s->part[fl][i] = Nfs[fl];
    }
}

static void state_copy(state_t* d, const state_t* s)
{
    state_init(d, s->Npt, s->Nfs);
    d->sign = s->sign;
    for (int fl = 0; fl < 2; ++fl) {
        memcpy(d->fock[fl], s->fock[fl], sizeof(int) * s->Nfs[fl]);
        memcpy(d->part[fl], s->part[fl], sizeof(int) * s->Npt[fl]);
    }
}

static void state_free(state_t* s)
{
    for (int fl = 0; fl < 2; ++fl) { free(s->fock[fl]); free(s->part[fl]); }
}

static int state_hopsign(const state_t* s, const hopset* h)   /* State.cpp:86-115 */
{
    int odd = 0;
    for (int fl = 0; fl < 2; ++fl) {
        if (h->n[fl]) {
            int a = h->from[fl], b = h->to[fl];
            int mn = (a < b ? a : b) + 1, mx = a > b ? a : b;
            for (int x = mn; x < mx; ++x) odd = (odd != (s->fock[fl][x] != s->Npt[fl]));
            if (h->n[fl] > 1) {
                /* the second hop counts on a copy with the first applied (State.cpp:97-110) */
                int* sf = (int*)malloc(sizeof(int) * s->Nfs[fl]);
                memcpy(sf, s->fock[fl], sizeof(int) * s->Nfs[fl]);
                int part = sf[a];
                sf[a] = s->Npt[fl];
                sf[b] = part;
                for (int hh = 1; hh < h->n[fl]; ++hh) {
                    int a2 = hop_from(h, fl, hh), b2 = hop_to(h, fl, hh);
                    int mn2 = (a2 < b2 ? a2 : b2) + 1, mx2 = a2 > b2 ? a2 : b2;
                    for (int x = mn2; x < mx2; ++x) odd = (odd != (sf[x] != s->Npt[fl]));
                    part = sf[a2];
                    if (part < s->Nfs[fl]) sf[part] = s->Npt[fl];   /* as State.cpp:107 writes it (by particle index) */
                    sf[b2] = part;
                }
                free(sf);
            }
        }
    }
    return 2 * (!odd) - 1;
}

static void state_hop(state_t* s, const hopset* h)   /* State.cpp:73-84 */
{
    s->sign *= state_hopsign(s, h);
    for (int fl = 0; fl < 2; ++fl)
        for (int hh = 0; hh < h->n[fl]; ++hh) {
            int f = hop_from(h, fl, hh), t = hop_to(h, fl, hh);
            int p = s->fock[fl][f];
            s->fock[fl][f] = s->Npt[fl];
            s->fock[fl][t] = p;
            s->part[fl][p] = t;
        }
}

static void state_initfock(state_t* s, int* const st[2])   /* State.cpp:29-41 */
{
    for (int fl = 0; fl < 2; ++fl) {
        int pi = 0;
        for (int x = 0; x < s->Nfs[fl]; ++x) {
            if (st[fl][x] < s->Npt[fl]) {
                s->fock[fl][x] = pi;
                s->part[fl][pi] = x;
                ++pi;
            }
        }
    }
}

/* get_hop_path (State.cpp:213-231), one hop per flavour at most. */
static int hop_path(const int* src, const int* dest, int n, int Npt, int* from, int* to)
{
    int np = 0, nh = 0, part[2] = {-1, -1}, hole[2] = {-1, -1};
    for (int x = 0; x < n; ++x) {
        if (src[x] == Npt && dest[x] != Npt) { if (np < 2) part[np] = x; ++np; }
        if (src[x] != Npt && dest[x] == Npt) { if (nh < 2) hole[nh] = x; ++nh; }
    }
    if (np > 2 || np != nh) return -1;
    for (int h = 0; h < 2; ++h) { from[h] = hole[h]; to[h] = part[h]; }   /* pairs in ascending order */
    return np;
}

/* ------------------------------------------------------------------ */
struct orc_job {
    int L, Ns, channel, qx, qy;
    double phi, neel, ne, bc[2];
    int N[2];
    int* fock2qn;      /* 3*Ns */
    int* qn2fock;      /* 2*Ns */
    zc* cache[2];      /* Ns*Ns: cache[fl][f*Ns + r] (WaveFunction.h:61-66) */
    int* nbr;          /* Ns*4 */
    int* deg;          /* Ns */
    int* edge_i;       /* 2*Ns */
    int* edge_j;
    int nedge;
    /* wavefunction states: exc[(i*Nexc + j)] hop set from state i to j */
    int Nexc;
    hopset* exc;
    state_t wav0;      /* wavefunction State after construction */
};

/* StagFluxWaveFunction::inmbz (StagFluxWaveFunction.cpp:89-101) */
static int sf_inmbz(const orc_job* j, int kx, int ky)
{
    double kkx = ((double)kx + j->bc[0] / 2.0) / (double)j->L;
    double kky = ((double)ky + j->bc[1] / 2.0) / (double)j->L;
    double eps = 1e-9;
    return (kkx >= 0 && kkx < 1 && kky >= 0 && kky < 1) &&
           (kkx + kky - 0.5 < 0 || kkx + kky - 1.5 >= -eps || kky - kkx - 0.5 > eps ||
            kky - kkx + 0.5 <= eps);
}

/* StagFluxWaveFunction::mbzmod (StagFluxWaveFunction.cpp:103-119) */
static void sf_mbzmod(const orc_job* j, int* k)
{
    int L = j->L;
    if (sf_inmbz(j, k[0], k[1])) return;
    if (k[0] < L / 2 && k[1] < L / 2) { k[0] += L / 2; k[1] += L / 2; }
    else if (k[0] < L / 2 && k[1] >= L / 2) { k[0] += L / 2; k[1] -= L / 2; }
    else if (k[0] >= L / 2 && k[1] < L / 2) { k[0] -= L / 2; k[1] += L / 2; }
    else { k[0] -= L / 2; k[1] -= L / 2; }
}

/* delta/neelk/omega/Uk/Vk (StagFluxWaveFunction.cpp:121-163) */
static zc sf_delta(const orc_job* j, const double* k)
{
    zc p1 = cplx(1.0 * cos(j->phi), 1.0 * sin(j->phi));      /* std::polar(1, phi) */
    zc p2 = cplx(1.0 * cos(-j->phi), 1.0 * sin(-j->phi));
    zc a = cos(k[0]) * p1;
    zc b = cos(k[1]) * p2;
    return 0.5 * (a + b);
}
static double sf_neelk(const orc_job* j, const double* k)
{
    if (j->ne == 0.0) return j->neel;
    return j->neel * pow(0.5 * (pow(cos(k[0]), 2.0) + pow(cos(k[1]), 2.0)), j->ne);
}
static double sf_omega(const orc_job* j, const double* k)
{
    zc d = sf_delta(j, k);
    double nd = creal(d) * creal(d) + cimag(d) * cimag(d);
    return sqrt(pow(sf_neelk(j, k), 2.0) + nd);
}
static zc cplx(double re, double im) { return CMPLX(re, im); }
static zc sf_Uk(const orc_job* j, const double* k, int up, int band)
{
    double om = sf_omega(j, k);
    zc d = sf_delta(j, k);
    double nk = sf_neelk(j, k);
    int sig = 2 * (!up) - 1;
    if (band == 0) return csqrt(0.5 * cplx(1 + sig * nk / om, 0.0));
    zc mc = cplx(-creal(d), cimag(d));      /* -conj(d) */
    double ad = cabs(d);
    zc q = cplx(creal(mc) / ad, cimag(mc) / ad);
    return q * csqrt(0.5 * cplx(1 - sig * nk / om, 0.0));
}
static zc sf_Vk(const orc_job* j, const double* k, int up, int band)
{
    double om = sf_omega(j, k);
    zc d = sf_delta(j, k);
    double nk = sf_neelk(j, k);
    int sig = 2 * (!up) - 1;
    if (band == 0) {
        double ad = cabs(d);
        zc q = cplx(creal(d) / ad, cimag(d) / ad);
        return q * csqrt(0.5 * cplx(1 - sig * nk / om, 0.0));
    }
    return csqrt(0.5 * cplx(1 + sig * nk / om, 0.0));
}

/* StagFluxWaveFunction::matrix_element (StagFluxWaveFunction.cpp:51-79) */
static zc sf_matrix_element(const orc_job* j, int fk, int fr, int up)
{
    double k[2], r[2];
    k[0] = ((double)j->fock2qn[3 * fk] + j->bc[0] / (2.0)) * 2 * M_PI / (double)j->L;
    k[1] = ((double)j->fock2qn[3 * fk + 1] + j->bc[1] / (2.0)) * 2 * M_PI / (double)j->L;
    r[1] = (double)(fr / j->L);
    r[0] = (double)fr - r[1] * (double)j->L;
    int band = j->fock2qn[3 * fk + 2];
    zc ph = cexp(cplx(0.0, k[0] * r[0] + k[1] * r[1]));
    zc s2 = cplx(sqrt(2.0) * creal(ph), sqrt(2.0) * cimag(ph));
    int par = (int)(r[0] + r[1]) % 2;
    zc u = sf_Uk(j, k, up, band), v = sf_Vk(j, k, up, band);
    zc a = cplx((double)(1 - par) * creal(u), (double)(1 - par) * cimag(u));
    zc b = cplx((double)par * creal(v), (double)par * cimag(v));
    zc out = s2 * (a + b);
    if (isnan(creal(out)) || isnan(cimag(out))) set_err(ORC_ERR_NAN);
    return out;
}

static zc matel(const orc_job* j, int f, int r, int fl) { return j->cache[fl][(size_t)f * j->Ns + r]; }

/* WaveFunction::AddState (WaveFunction.cpp:39-67) restated over an array of
 * per-flavour Fock vectors (value Npt = empty). */
static int wav_add_states(orc_job* j, int nst, int** st /* nst*2 vectors of Ns */)
{
    j->Nexc = nst;
    j->exc = (hopset*)calloc((size_t)nst * nst, sizeof(hopset));
    int Npt[2] = {j->N[0], j->N[1]};
    int Nfs[2] = {j->Ns, j->Ns};
    state_init(&j->wav0, Npt, Nfs);
    for (int fl = 0; fl < 2; ++fl) {
        int sti = 0;
        for (int x = 0; x < j->Ns; ++x)
            if (st[0 * 2 + fl][x] != Npt[fl]) { j->wav0.fock[fl][x] = sti; j->wav0.part[fl][sti] = x; ++sti; }
    }
    int* state = (int*)malloc(sizeof(int) * j->Ns);
    for (int a = 1; a < nst; ++a) {
        for (int fl = 0; fl < 2; ++fl) {
            for (int i = 0; i < a; ++i) {
                /* get_hop_state(m_exc[0][i][fl], m_fock[fl], ...) (State.cpp:233-244) */
                memcpy(state, j->wav0.fock[fl], sizeof(int) * j->Ns);
                const hopset* h0 = &j->exc[0 * nst + i];
                for (int hh = 0; hh < h0->n[fl]; ++hh) {
                    int f = hop_from(h0, fl, hh), t = hop_to(h0, fl, hh);
                    state[t] = state[f];
                    state[f] = Npt[fl];
                }
                hopset* ha = &j->exc[a * nst + i];
                hopset* hb = &j->exc[i * nst + a];
                int f1[2], t1[2], f2[2], t2[2];
                int n1 = hop_path(st[a * 2 + fl], state, j->Ns, Npt[fl], f1, t1);
                int n2 = hop_path(state, st[a * 2 + fl], j->Ns, Npt[fl], f2, t2);
                if (n1 < 0 || n2 < 0) { free(state); return ORC_ERR_INVALID; }
                ha->n[fl] = n1; ha->from[fl] = f1[0]; ha->to[fl] = t1[0]; ha->from2[fl] = f1[1]; ha->to2[fl] = t1[1];
                hb->n[fl] = n2; hb->from[fl] = f2[0]; hb->to[fl] = t2[0]; hb->from2[fl] = f2[1]; hb->to2[fl] = t2[1];
            }
        }
    }
    free(state);
    return ORC_OK;
}

orc_job* orc_job_create(int L, double phi, double neel, double neel_exp,
                        double bcx, double bcy, int channel, int qx, int qy, int* status)
{
    tl_err = 0;
    if (L < 2 || (L * L) % 2 || channel < 0 || channel > 2) { if (status) *status = ORC_ERR_INVALID; return NULL; }
    orc_job* j = (orc_job*)calloc(1, sizeof(orc_job));
    j->L = L; j->Ns = L * L; j->channel = channel; j->qx = qx; j->qy = qy;
    j->phi = phi; j->neel = neel; j->ne = neel_exp; j->bc[0] = bcx; j->bc[1] = bcy;
    int Ns = j->Ns;
    if (channel == ORC_CH_TRANS) { j->N[0] = Ns / 2 + 1; j->N[1] = Ns / 2 - 1; }
    else { j->N[0] = Ns / 2; j->N[1] = Ns / 2; }
    /* MBZ enumeration (StagFluxWaveFunction.cpp:24-41) */
    j->fock2qn = (int*)calloc(3 * (size_t)Ns + 6, sizeof(int));
    j->qn2fock = (int*)malloc(sizeof(int) * 2 * Ns);
    for (int i = 0; i < 2 * Ns; ++i) j->qn2fock[i] = Ns;
    int idx = 0;
    for (int kx = 0; kx < L; ++kx)
        for (int ky = 0; ky < L; ++ky)
            if (sf_inmbz(j, kx, ky)) {
                if (idx + 1 >= Ns + 1) { idx += 2; continue; }
                j->fock2qn[idx * 3] = kx; j->fock2qn[idx * 3 + 1] = ky; j->fock2qn[idx * 3 + 2] = 0;
                j->qn2fock[(kx * L + ky) * 2] = idx; idx++;
                j->fock2qn[idx * 3] = kx; j->fock2qn[idx * 3 + 1] = ky; j->fock2qn[idx * 3 + 2] = 1;
                j->qn2fock[(kx * L + ky) * 2 + 1] = idx; idx++;
            }
    if (idx != Ns) { orc_job_destroy(j); if (status) *status = ORC_ERR_INVALID; return NULL; }
    /* Φ cache (WaveFunction.cpp:27-37) */
    for (int fl = 0; fl < 2; ++fl) {
        j->cache[fl] = (zc*)malloc(sizeof(zc) * (size_t)Ns * Ns);
        for (int f = 0; f < Ns; ++f)
            for (int r = 0; r < Ns; ++r) j->cache[fl][(size_t)f * Ns + r] = sf_matrix_element(j, f, r, fl);
    }
    /* SquareLattice (SquareLattice.cpp:9-28) and Edge (Lattice.h:24-41):
     * edges appended to both endpoints' lists in creation order. */
    j->nedge = 2 * Ns;
    j->edge_i = (int*)malloc(sizeof(int) * j->nedge);
    j->edge_j = (int*)malloc(sizeof(int) * j->nedge);
    j->nbr = (int*)malloc(sizeof(int) * 4 * Ns);
    j->deg = (int*)calloc(Ns, sizeof(int));
    int e = 0;
    for (int x = 0; x < L; ++x)
        for (int y = 0; y < L; ++y) {
            int a = y * L + x;
            int b1 = ((y + 1) % L) * L + x;
            int b2 = y * L + (x + 1) % L;
            int pairs[2][2] = {{a, b1}, {a, b2}};
            for (int q = 0; q < 2; ++q) {
                int u = pairs[q][0], v = pairs[q][1];
                j->edge_i[e] = u; j->edge_j[e] = v; ++e;
                if (j->deg[u] < 4) j->nbr[u * 4 + j->deg[u]] = v;
                j->deg[u]++;
                if (j->deg[v] < 4) j->nbr[v * 4 + j->deg[v]] = u;
                j->deg[v]++;
            }
        }
    /* Channel states */
    int rc = ORC_OK;
    if (channel == ORC_CH_GROUNDSTATE) {   /* StagFluxGroundState.cpp:3-15 */
        int* fst = (int*)malloc(sizeof(int) * Ns);
        for (int x = 0; x < Ns; ++x) fst[x] = Ns / 2;
        for (int f = 0; f < Ns / 2; ++f) fst[2 * f] = f;
        int* st[2] = {fst, fst};
        rc = wav_add_states(j, 1, st);
        free(fst);
    } else if (channel == ORC_CH_TRANS) {  /* StagFluxTransExciton.cpp:7-44 */
        int nst = Ns / 2;
        int** st = (int**)malloc(sizeof(int*) * 2 * nst);
        for (int fe = 0; fe < nst; ++fe) {
            int kx = j->fock2qn[3 * (2 * fe + 1)], ky = j->fock2qn[3 * (2 * fe + 1) + 1];
            int Qk[2] = {((kx - qx) % L + L) % L, ((ky - qy) % L + L) % L};
            sf_mbzmod(j, Qk);
            int* s0 = (int*)malloc(sizeof(int) * Ns);
            int* s1 = (int*)malloc(sizeof(int) * Ns);
            for (int x = 0; x < Ns; ++x) { s0[x] = Ns / 2 + 1; s1[x] = Ns / 2 - 1; }
            int dc = 0;
            for (int f = 0; f < Ns / 2; ++f) {
                s0[2 * f] = f;
                if (j->qn2fock[(Qk[0] * L + Qk[1]) * 2] != 2 * f) { s1[2 * f] = dc; ++dc; }
            }
            s0[2 * fe + 1] = Ns / 2;
            st[fe * 2 + 0] = s0; st[fe * 2 + 1] = s1;
        }
        rc = wav_add_states(j, nst, st);
        for (int i = 0; i < 2 * nst; ++i) free(st[i]);
        free(st);
    } else {                               /* StagFluxLongExciton.cpp:6-66 */
        int extra = ((qx == 0 && qy == 0) || (qx == L / 2 && qy == L / 2)) ? 1 : 0;
        int nst = Ns + extra;
        int** st = (int**)malloc(sizeof(int*) * 2 * nst);
        int a = 0;
        for (int fe = 0; fe < Ns / 2; ++fe) {
            int kx = j->fock2qn[3 * (2 * fe + 1)], ky = j->fock2qn[3 * (2 * fe + 1) + 1];
            int Qk[2] = {((kx - qx) % L + L) % L, ((ky - qy) % L + L) % L};
            sf_mbzmod(j, Qk);
            for (int which = 0; which < 2; ++which) {
                int* s0 = (int*)malloc(sizeof(int) * Ns);
                int* s1 = (int*)malloc(sizeof(int) * Ns);
                for (int x = 0; x < Ns; ++x) { s0[x] = Ns / 2; s1[x] = Ns / 2; }
                int* full = which == 0 ? s1 : s0;
                int* holed = which == 0 ? s0 : s1;
                int cnt = 0;
                for (int f = 0; f < Ns / 2; ++f) {
                    full[2 * f] = f;
                    if (j->qn2fock[(Qk[0] * L + Qk[1]) * 2] != 2 * f) { holed[2 * f] = cnt; ++cnt; }
                }
                holed[2 * fe + 1] = Ns / 2 - 1;
                st[a * 2 + 0] = s0; st[a * 2 + 1] = s1; ++a;
            }
        }
        if (extra) {
            int* s0 = (int*)malloc(sizeof(int) * Ns);
            int* s1 = (int*)malloc(sizeof(int) * Ns);
            for (int x = 0; x < Ns; ++x) { s0[x] = Ns / 2; s1[x] = Ns / 2; }
            for (int f = 0; f < Ns / 2; ++f) { s0[2 * f] = f; s1[2 * f] = f; }
            st[a * 2 + 0] = s0; st[a * 2 + 1] = s1; ++a;
        }
        rc = wav_add_states(j, nst, st);
        for (int i = 0; i < 2 * nst; ++i) free(st[i]);
        free(st);
    }
    if (!rc && tl_err) rc = tl_err;
    if (rc) { orc_job_destroy(j); if (status) *status = rc; return NULL; }
    if (status) *status = ORC_OK;
    return j;
}

void orc_job_destroy(orc_job* j)
{
    if (!j) return;
    free(j->fock2qn); free(j->qn2fock);
    free(j->cache[0]); free(j->cache[1]);
    free(j->nbr); free(j->deg); free(j->edge_i); free(j->edge_j);
    if (j->exc) { free(j->exc); state_free(&j->wav0); }
    free(j);
}

void orc_job_info(const orc_job* j, int* Ns, int* Nup, int* Ndn, int* Nexc)
{
    if (Ns) *Ns = j->Ns;
    if (Nup) *Nup = j->N[0];
    if (Ndn) *Ndn = j->N[1];
    if (Nexc) *Nexc = j->Nexc;
}

void orc_job_phi(const orc_job* j, int fl, double* out)
{
    size_t n = (size_t)j->Ns * j->Ns;
    for (size_t i = 0; i < n; ++i) { out[2 * i] = creal(j->cache[fl][i]); out[2 * i + 1] = cimag(j->cache[fl][i]); }
}

void orc_job_neighbours(const orc_job* j, int32_t* nbr)
{
    for (int i = 0; i < 4 * j->Ns; ++i) nbr[i] = j->nbr[i];
}

void orc_job_orbitals(const orc_job* j, int fl, int32_t* orb)
{
    for (int p = 0; p < j->N[fl]; ++p) orb[p] = j->wav0.part[fl][p];
}

/* ------------------------------------------------------------------ */
struct orc_walker {
    orc_job* j;
    state_t lat;       /* LatticeState */
    state_t wav;       /* WaveFunction's State part */
    int cur;           /* m_c_exc */
    zc* mat[2];        /* m_mat, column-major N x N: A(f, r) at [r*N + f] */
    zc* mati[2];       /* m_mati */
    bigc amp;          /* m_amp */
    int amp_ok;
    /* LatticeStepper (LatticeStepper.h:16-37) */
    hopset prev;
    int khop;
    bigd prev_weight, weight;
    /* MetroMC (MetroMC.h:11-45) */
    bigd state_weight;
    uint64_t steps, rejection;
    uint64_t accepted_real, reinversions, since_reinv;
    rng_t rng;
    /* quantities */
    int meas_pj, meas_sm, meas_ss;
    bigc* pj;          /* unused placeholder */
    zc* pj_vals;       /* 2*Nexc*Nexc */
    zc sm_val;
    zc* ss_vals;       /* 5*Ns*Ns */
    zc* work;          /* scratch */
};

static int wav_hopsign(const orc_walker* w, const hopset* h) { return state_hopsign(&w->wav, h); }
static const hopset* wav_gethops(const orc_walker* w) { return &w->j->exc[(size_t)w->cur * w->j->Nexc]; }
static void wav_hop(orc_walker* w, int k)   /* WaveFunction.cpp:69-73 */
{
    state_hop(&w->wav, &w->j->exc[(size_t)w->cur * w->j->Nexc + k]);
    w->cur = k;
}

/* linalg::DetInv (linalg.cpp:9-44) with zgetrf/zgetri written out. */
static int lu_factor(zc* a, int n, int* ipiv)
{
    for (int j = 0; j < n; ++j) {
        int p = j;
        double best = -1.0;
        for (int i = j; i < n; ++i) {
            double v = fabs(creal(a[i + (size_t)j * n])) + fabs(cimag(a[i + (size_t)j * n]));
            if (v > best) { best = v; p = i; }
        }
        ipiv[j] = p + 1;
        if (creal(a[p + (size_t)j * n]) != 0.0 || cimag(a[p + (size_t)j * n]) != 0.0) {
            if (p != j)
                for (int c = 0; c < n; ++c) {
                    zc t = a[j + (size_t)c * n]; a[j + (size_t)c * n] = a[p + (size_t)c * n]; a[p + (size_t)c * n] = t;
                }
            zc r = 1.0 / a[j + (size_t)j * n];
            for (int i = j + 1; i < n; ++i) a[i + (size_t)j * n] *= r;
        }
        for (int c = j + 1; c < n; ++c) {
            zc t = a[j + (size_t)c * n];
            if (creal(t) != 0.0 || cimag(t) != 0.0)
                for (int i = j + 1; i < n; ++i) a[i + (size_t)c * n] -= a[i + (size_t)j * n] * t;
        }
    }
    return 0;
}

static void lu_inverse(zc* a, int n, const int* ipiv, zc* work)
{
    /* inv(U) in place (ztrti2, upper, non-unit) */
    for (int j = 0; j < n; ++j) {
        a[j + (size_t)j * n] = 1.0 / a[j + (size_t)j * n];
        zc ajj = -a[j + (size_t)j * n];
        for (int k = 0; k < j; ++k) {           /* x = triu(A[0:j,0:j]) * x */
            zc t = a[k + (size_t)j * n];
            if (creal(t) != 0.0 || cimag(t) != 0.0) {
                for (int i = 0; i < k; ++i) a[i + (size_t)j * n] += t * a[i + (size_t)k * n];
                a[k + (size_t)j * n] = t * a[k + (size_t)k * n];
            }
        }
        for (int i = 0; i < j; ++i) a[i + (size_t)j * n] *= ajj;
    }
    /* solve inv(A)*L = inv(U) */
    for (int j = n - 1; j >= 0; --j) {
        for (int i = j + 1; i < n; ++i) { work[i] = a[i + (size_t)j * n]; a[i + (size_t)j * n] = 0.0; }
        if (j < n - 1)
            for (int c = j + 1; c < n; ++c) {
                zc t = work[c];
                for (int i = 0; i < n; ++i) a[i + (size_t)j * n] -= a[i + (size_t)c * n] * t;
            }
    }
    for (int j = n - 2; j >= 0; --j) {
        int jp = ipiv[j] - 1;
        if (jp != j)
            for (int i = 0; i < n; ++i) {
                zc t = a[i + (size_t)j * n]; a[i + (size_t)j * n] = a[i + (size_t)jp * n]; a[i + (size_t)jp * n] = t;
            }
    }
}

static int det_inv(const zc* A, zc* Ii, int M, bigc* d, zc* work)
{
    int* ipiv = (int*)malloc(sizeof(int) * (M > 0 ? M : 1));
    memcpy(Ii, A, sizeof(zc) * (size_t)M * M);
    lu_factor(Ii, M, ipiv);
    int perm = 1;
    for (int i = 0; i < M; ++i) if (ipiv[i] != i + 1) perm *= -1;
    *d = bigc_make((double)perm, 0);
    for (int i = 0; i < M; ++i) bigc_muleq(d, bigc_make(Ii[(size_t)i * M + i], 0));
    int singular = bigd_d(bigc_norm(*d)) < 1e-9;
    if (!singular) lu_inverse(Ii, M, ipiv, work);
    else *d = bigc_make(0.0, 0);
    free(ipiv);
    return singular;
}

/* linalg::Det for M <= 2 (linalg.cpp:46-58) */
static bigc det_small(const zc* B, int M)
{
    if (M == 0) return bigc_make(1.0, 0);
    if (M == 1) return bigc_make(B[0], 0);
    return bigc_make(B[0] * B[3] - B[1] * B[2], 0);
}

/* The plain-loop BLAS the reference build links (zgemm 'N','N', zgemv 'N',
 * zgeru, zdotu), in the same loop order, for the rank-2 row branches. */
static void zgemm_nn(int m, int n, int k, zc alpha, const zc* a, int lda, const zc* b, int ldb, zc beta, zc* c,
                     int ldc)
{
    for (int jj = 0; jj < n; ++jj) {
        for (int i = 0; i < m; ++i) {
            zc* cij = &c[i + (size_t)jj * ldc];
            *cij = (creal(beta) == 0.0 && cimag(beta) == 0.0) ? 0.0 : beta * *cij;
        }
        for (int l = 0; l < k; ++l) {
            zc t = alpha * b[l + (size_t)jj * ldb];
            for (int i = 0; i < m; ++i) c[i + (size_t)jj * ldc] += t * a[i + (size_t)l * lda];
        }
    }
}

static void zgemv_n(int m, int n, zc alpha, const zc* a, int lda, const zc* x, int incx, zc beta, zc* y, int incy)
{
    for (int i = 0; i < m; ++i) {
        zc* yi = &y[(size_t)i * incy];
        *yi = (creal(beta) == 0.0 && cimag(beta) == 0.0) ? 0.0 : beta * *yi;
    }
    for (int jj = 0; jj < n; ++jj) {
        zc t = alpha * x[(size_t)jj * incx];
        for (int i = 0; i < m; ++i) y[(size_t)i * incy] += t * a[i + (size_t)jj * lda];
    }
}

static void zgeru_(int m, int n, zc alpha, const zc* x, int incx, const zc* y, int incy, zc* a, int lda)
{
    for (int jj = 0; jj < n; ++jj) {
        zc t = alpha * y[(size_t)jj * incy];
        for (int i = 0; i < m; ++i) a[i + (size_t)jj * lda] += x[(size_t)i * incx] * t;
    }
}

static zc zdotu(int n, const zc* x, int incx, const zc* y, int incy)
{
    zc s = 0.0;
    for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
    return s;
}

/* linalg::Det (linalg.cpp:46-73): closed forms up to M = 2, LU (zgetrf) above */
static bigc det_any(const zc* B, int M)
{
    if (M <= 2) return det_small(B, M);
    zc* AA = (zc*)malloc(sizeof(zc) * (size_t)M * M);
    int* ipiv = (int*)malloc(sizeof(int) * M);
    memcpy(AA, B, sizeof(zc) * (size_t)M * M);
    lu_factor(AA, M, ipiv);
    int perm = 1;
    for (int i = 0; i < M; ++i) if (ipiv[i] != i + 1) perm *= -1;
    bigc d = bigc_make((double)perm, 0);
    for (int i = 0; i < M; ++i) bigc_muleq(&d, bigc_make(AA[(size_t)i * M + i], 0));
    free(AA);
    free(ipiv);
    return d;
}

/* DetUpdate's B for one column (rc0 <= 1) and two rows of hop set r
 * (linalg.cpp:139-258, the rr[r] > 1 arms). */
static bigc det_update_rows2(const zc* A, const zc* Ai, int N, const zc* C, const int* ci, int rc0, zc EcAiC,
                             const zc* RAiC, int Nr, const zc* R, int ldr, const int* ri, int rid)
{
    const int rr = 2, m = rc0 + rr;
    zc B[9] = {0};
    zc ErTAEcT[2] = {0, 0}, ErTC[2] = {0, 0};
    for (int i = 0; i < rr; ++i)                       /* B22: zdotu R row . Ai column */
        for (int jj = 0; jj < rr; ++jj)
            B[rc0 + i + (size_t)(rc0 + jj) * m] = zdotu(N, &R[rid + i], ldr, &Ai[(size_t)ri[rid + jj] * N], 1);
    if (rc0) B[0] = EcAiC;                             /* B11 */
    if (rc0) {
        for (int jj = 0; jj < rr; ++jj) B[(size_t)(rc0 + jj) * m] = Ai[ci[0] + (size_t)ri[rid + jj] * N];   /* B12 */
        for (int i = 0; i < rr; ++i) {
            ErTAEcT[i] = A[ri[rid + i] + (size_t)ci[0] * N];
            ErTC[i] = C[ri[rid + i]];
            B[rc0 + i] = RAiC[rid + i] - R[rid + i + (size_t)ci[0] * ldr];                             /* B21 */
        }
        zgemv_n(rr, rr, 1.0, &B[rc0 * m + rc0], m, ErTAEcT, 1, 1.0, &B[rc0], 1);
        zgemv_n(rr, rr, 1.0, &B[rc0 * m + rc0], m, ErTC, 1, 1.0, &B[rc0], 1);
        zc mem = zdotu(rr, &B[rc0 * m], m, ErTC, 1);
        B[0] += mem;
        mem = zdotu(rr, &B[rc0 * m], m, ErTAEcT, 1);
        B[0] += mem;
    }
    (void)Nr;
    return det_any(B, m);
}

/* DetUpdate's nr <= 1 branch with a two-row hop set (linalg.cpp:259-378, the
 * rr[0] > 1 arms): one B per column hop set c. */
static int det_update_cols_rows2(const zc* A, const zc* Ai, int N, const zc* C, int ldc, const int* ci,
                                 const int* rc, int nc, const zc* R, int ldr, const int* ri, int nr, bigc* dets)
{
    const int rr = 2;
    int* cid = (int*)malloc(sizeof(int) * nc);
    int Nc = 0;
    for (int c = 0; c < nc; ++c) { cid[c] = Nc; Nc += rc[c]; }
    zc* RAi = (zc*)malloc(sizeof(zc) * rr * (size_t)N);
    zc* RAiC = (zc*)malloc(sizeof(zc) * rr * (size_t)(Nc > 0 ? Nc : 1));
    zc RAiEr[4];
    zgemm_nn(rr, N, N, 1.0, R, ldr, Ai, N, 0.0, RAi, rr);                 /* R * Ai */
    for (int i = 0; i < rr; ++i)
        for (int jj = 0; jj < rr; ++jj) RAiEr[jj * rr + i] = RAi[i + (size_t)ri[jj] * rr];
    if (Nc) zgemm_nn(rr, Nc, N, 1.0, RAi, rr, C, ldc, 0.0, RAiC, rr);     /* R * Ai * C */
    for (int c = 0; c < nc; ++c) {
        const int m = rc[c] + rr;
        zc B[9] = {0};
        zc ErTAEcT[2] = {0, 0}, REcT[2] = {0, 0};
        if (rc[c]) B[0] = zdotu(N, &Ai[ci[cid[c]]], N, &C[(size_t)cid[c] * ldc], 1);   /* B11 */
        for (int i = 0; i < rr; ++i)                                                   /* B22 */
            for (int jj = 0; jj < rr; ++jj) B[(size_t)(rc[c] + jj) * m + rc[c] + i] = RAiEr[jj * rr + i];
        if (rc[c]) {
            for (int jj = 0; jj < rr; ++jj) B[(size_t)(rc[c] + jj) * m] = Ai[ci[cid[c]] + (size_t)ri[jj] * N];   /* B12 */
            for (int i = 0; i < rr; ++i) {
                ErTAEcT[i] = A[ri[i] + (size_t)ci[cid[c]] * N];
                REcT[i] = R[i + (size_t)ci[cid[c]] * nr * rr];          /* row stride as linalg.cpp:322 */
                B[rc[c] + i] = RAiC[i + (size_t)cid[c] * rr] - C[ri[i] + (size_t)cid[c] * ldc];   /* B21 */
            }
            for (int i = 0; i < rr; ++i) B[rc[c] + i] += (ErTAEcT[i] + REcT[i]) * B[0];
            zgeru_(rr, rr, 1.0, REcT, 1, &B[(size_t)rc[c] * m], m, &B[(size_t)rc[c] * m + rc[c]], m);
            zgeru_(rr, rr, 1.0, ErTAEcT, 1, &B[(size_t)rc[c] * m], m, &B[(size_t)rc[c] * m + rc[c]], m);
        }
        dets[c] = det_any(B, m);
    }
    free(cid);
    free(RAi);
    free(RAiC);
    return ORC_OK;
}

/* linalg::DetUpdate (linalg.cpp:107-400), ranks rc in {0,1}, rr in {0,1,2}. */
static int det_update(const zc* A, const zc* Ai, int N, const zc* C, int ldc, const int* ci,
                      const int* rc, int nc, const zc* R, int ldr, const int* ri, const int* rr,
                      int nr, bigc* dets, zc* work)
{
    for (int c = 0; c < nc; ++c) if (rc[c] > 1) return ORC_ERR_INVALID;
    for (int r = 0; r < nr; ++r) if (rr[r] > 2) return ORC_ERR_INVALID;
    if (nc > 1 && nr <= 1 && nr && rr[0] == 2)
        return det_update_cols_rows2(A, Ai, N, C, ldc, ci, rc, nc, R, ldr, ri, nr, dets);
    if (nc <= 1) {
        int* rid = (int*)malloc(sizeof(int) * (nr > 0 ? nr : 1));
        int Nr = 0;
        for (int r = 0; r < nr; ++r) { rid[r] = Nr; Nr += rr[r]; }
        zc* AiC = work;              /* N */
        zc* RAiC = (zc*)malloc(sizeof(zc) * (Nr > 0 ? Nr : 1));
        zc EcAiC = 0.0;
        int rc0 = nc ? rc[0] : 0;
        if (nc && rc0) {
            for (int i = 0; i < N; ++i) AiC[i] = 0.0;
            for (int jj = 0; jj < N; ++jj) {          /* zgemv 'N' */
                zc t = C[jj];
                for (int i = 0; i < N; ++i) AiC[i] += t * Ai[i + (size_t)jj * N];
            }
            EcAiC = AiC[ci[0]];
            if (Nr)
                for (int i = 0; i < Nr; ++i) {         /* zgemv 'N' Nr x N, lda = ldr */
                    zc s = 0.0;
                    for (int jj = 0; jj < N; ++jj) s += R[i + (size_t)jj * ldr] * AiC[jj];
                    RAiC[i] = s;
                }
        }
        for (int r = 0; r < nr; ++r) {
            if (rr[r] == 2) {
                dets[r] = det_update_rows2(A, Ai, N, C, ci, nc ? rc0 : 0, EcAiC, RAiC, Nr, R, ldr, ri, rid[r]);
                continue;
            }
            zc B[4] = {0, 0, 0, 0};
            int m = rc0 + rr[r];
            if (rr[r]) {                                /* zdotu R row . Ai column ri */
                zc s = 0.0;
                const zc* x = &R[rid[r]];
                const zc* y = &Ai[(size_t)ri[rid[r]] * N];
                for (int k = 0; k < N; ++k) s += x[(size_t)k * ldr] * y[k];
                B[rc0 + rc0 * m] = s;
            }
            if (rc0) B[0] = EcAiC;
            if (nc && rc0 && rr[r]) {
                B[m] = Ai[ci[0] + (size_t)ri[rid[r]] * N];            /* B12 */
                zc ErTAEcT = A[ri[rid[r]] + (size_t)ci[0] * N];
                zc ErTC = C[ri[rid[r]]];
                B[1] = RAiC[rid[r]] - R[rid[r] + (size_t)ci[0] * ldr];  /* B21 */
                B[1] += B[3] * (ErTAEcT + ErTC);
                B[0] += B[2] * (ErTC + ErTAEcT);
            }
            dets[r] = det_small(B, m);
        }
        free(rid);
        free(RAiC);
        return ORC_OK;
    } else if (nr <= 1) {
        int* cid = (int*)malloc(sizeof(int) * nc);
        int Nc = 0;
        for (int c = 0; c < nc; ++c) { cid[c] = Nc; Nc += rc[c]; }
        int rr0 = nr ? rr[0] : 0;
        zc* RAi = work;          /* N */
        zc* RAiC = (zc*)malloc(sizeof(zc) * (Nc > 0 ? Nc : 1));
        zc RAiEr = 0.0;
        if (nr && rr0) {
            for (int jj = 0; jj < N; ++jj) {            /* zgemv 'T' */
                zc s = 0.0;
                for (int i = 0; i < N; ++i) s += Ai[i + (size_t)jj * N] * R[(size_t)i * ldr];
                RAi[jj] = s;
            }
            RAiEr = RAi[ri[0]];
            for (int c = 0; c < Nc; ++c) {              /* zgemv 'T' N x Nc */
                zc s = 0.0;
                for (int i = 0; i < N; ++i) s += C[i + (size_t)c * ldc] * RAi[i];
                RAiC[c] = s;
            }
        }
        for (int c = 0; c < nc; ++c) {
            zc B[4] = {0, 0, 0, 0};
            int m = rc[c] + rr0;
            if (rc[c]) {                                 /* zdotu Ai row ci . C column */
                zc s = 0.0;
                const zc* x = &Ai[ci[cid[c]]];
                const zc* y = &C[(size_t)cid[c] * ldc];
                for (int k = 0; k < N; ++k) s += x[(size_t)k * N] * y[k];
                B[0] = s;
            }
            if (rr0) B[rc[c] + rc[c] * m] = RAiEr;
            if (rr0 && rc[c]) {
                B[m] = Ai[ci[cid[c]] + (size_t)ri[0] * N];              /* B12 */
                zc ErTAEcT = A[ri[0] + (size_t)ci[cid[c]] * N];
                zc REcT = R[(size_t)ci[cid[c]] * nr * rr0];             /* stride as linalg.cpp:322 */
                B[1] = RAiC[cid[c] * rr0] - C[ri[0] + (size_t)cid[c] * ldc];
                B[1] += (ErTAEcT + REcT) * B[0];
                B[3] += (REcT + ErTAEcT) * B[2];
            }
            dets[c] = det_small(B, m);
        }
        free(cid);
        free(RAiC);
        return ORC_OK;
    }
    return ORC_ERR_INVALID;
}

/* linalg::InvUpdate (linalg.cpp:402-573) as written there, through the
 * plain-loop zgemm: used for two row changes (R is rr x N with leading
 * dimension rr, C is N x rc). */
static int inv_update_general(const zc* A, zc* Ai, int N, const zc* C, const int* ci, int rc,
                              const zc* R, const int* ri, int rr, bigc* det)
{
    const int m = rc + rr;
    const zc one = 1.0, zer = 0.0, mone = -1.0;
    zc* EcAiC = (zc*)calloc((size_t)rc * rc + 1, sizeof(zc));
    zc* RAiEr = (zc*)calloc((size_t)rr * rr + 1, sizeof(zc));
    zc* B = (zc*)calloc((size_t)m * m, sizeof(zc));
    zc* Bi = (zc*)calloc((size_t)m * m, sizeof(zc));
    zc* RAiC = (zc*)calloc((size_t)rr * rc + 1, sizeof(zc));
    zc* ErTAEcT = (zc*)calloc((size_t)rr * rc + 1, sizeof(zc));
    zc* ErTC = (zc*)calloc((size_t)rr * rc + 1, sizeof(zc));
    zc* REcT = (zc*)calloc((size_t)rr * rc + 1, sizeof(zc));
    zc* AiC = (zc*)calloc((size_t)N * rc + 1, sizeof(zc));
    zc* EcAi = (zc*)calloc((size_t)rc * N + 1, sizeof(zc));
    zc* RAi = (zc*)calloc((size_t)rr * N + 1, sizeof(zc));
    zc* AiEr = (zc*)calloc((size_t)N * rr + 1, sizeof(zc));
    zc* mem = (zc*)calloc((size_t)(rc > rr ? rc : rr) * N + 1, sizeof(zc));
    zc* lu = (zc*)calloc((size_t)m + 1, sizeof(zc));
    if (rc) zgemm_nn(N, rc, N, one, Ai, N, C, N, zer, AiC, N);
    if (rr) zgemm_nn(rr, N, N, one, R, rr, Ai, N, zer, RAi, rr);
    for (int i = 0; i < rc; ++i)
        for (int jj = 0; jj < rc; ++jj) EcAiC[jj * rc + i] = AiC[ci[i] + (size_t)jj * N];
    for (int i = 0; i < rr; ++i)
        for (int jj = 0; jj < rr; ++jj) RAiEr[i + jj * rr] = RAi[i + (size_t)ri[jj] * rr];
    if (rc * rr) zgemm_nn(rr, rc, N, one, RAi, rr, C, N, zer, RAiC, rr);
    for (int i = 0; i < rr; ++i)
        for (int jj = 0; jj < rc; ++jj) {
            ErTAEcT[i + jj * rr] = A[ri[i] + (size_t)ci[jj] * N];
            ErTC[i + jj * rr] = C[ri[i] + (size_t)jj * N];
            REcT[i + jj * rr] = R[i + (size_t)ci[jj] * rr];
        }
    for (int i = 0; i < rc; ++i)
        for (int jj = 0; jj < rr; ++jj) B[i + (size_t)(rc + jj) * m] = Ai[ci[i] + (size_t)ri[jj] * N];   /* B12 */
    for (int i = 0; i < rr; ++i)
        for (int jj = 0; jj < rr; ++jj) B[(rc + i) + (size_t)(rc + jj) * m] = RAiEr[i + jj * rr];       /* B22 */
    for (int i = 0; i < rc; ++i)
        for (int jj = 0; jj < rc; ++jj) B[i + (size_t)jj * m] = EcAiC[i + jj * rc];                   /* B11 */
    if (rr * rc) {
        zgemm_nn(rc, rc, rr, mone, &B[(size_t)rc * m], m, ErTC, rr, one, B, m);
        zgemm_nn(rc, rc, rr, one, &B[(size_t)rc * m], m, ErTAEcT, rr, one, B, m);
    }
    for (int i = 0; i < rr; ++i)
        for (int jj = 0; jj < rc; ++jj) B[(rc + i) + (size_t)jj * m] = RAiC[i + jj * rr] - R[i + (size_t)ci[jj] * rr];
    if (rr * rc) {
        zgemm_nn(rr, rc, rr, one, &B[(size_t)rc * m + rc], m, ErTAEcT, rr, one, &B[rc], m);
        zgemm_nn(rr, rc, rr, mone, &B[(size_t)rc * m + rc], m, ErTC, rr, one, &B[rc], m);
    }
    int st = ORC_OK;
    if (!det_inv(B, Bi, m, det, lu)) {
        for (int i = 0; i < N; ++i) {
            for (int jj = 0; jj < rr; ++jj) AiEr[i + (size_t)jj * N] = Ai[i + (size_t)ri[jj] * N];
            for (int jj = 0; jj < rc; ++jj) EcAi[jj + (size_t)i * rc] = Ai[ci[jj] + (size_t)i * N];
        }
        if (rr * rc) {
            zgemm_nn(N, rc, rr, mone, AiEr, N, ErTC, rr, one, AiC, N);
            zgemm_nn(N, rc, rr, one, AiEr, N, ErTAEcT, rr, one, AiC, N);
        }
        for (int c = 0; c < rc; ++c) AiC[ci[c] + (size_t)c * N] -= 1;
        for (int r = 0; r < rr; ++r) RAi[r + (size_t)ri[r] * rr] -= 1;
        if (rc) {
            zgemm_nn(rc, N, rc, one, Bi, m, EcAi, rc, zer, mem, rc);
            zgemm_nn(N, N, rc, mone, AiC, N, mem, rc, one, Ai, N);
        }
        if (rc * rr) {
            zgemm_nn(rc, N, rr, one, &Bi[(size_t)rc * m], m, RAi, rr, zer, mem, rc);
            zgemm_nn(N, N, rc, mone, AiC, N, mem, rc, one, Ai, N);
            zgemm_nn(rr, N, rc, one, &Bi[rc], m, EcAi, rc, zer, mem, rr);
            zgemm_nn(N, N, rr, mone, AiEr, N, mem, rr, one, Ai, N);
        }
        if (rr) {
            zgemm_nn(rr, N, rr, one, &Bi[(size_t)rc * m + rc], m, RAi, rr, zer, mem, rr);
            zgemm_nn(N, N, rr, mone, AiEr, N, mem, rr, one, Ai, N);
        }
    } else {
        st = ORC_ERR_SINGULAR;
    }
    free(EcAiC); free(RAiEr); free(B); free(Bi); free(RAiC); free(ErTAEcT); free(ErTC); free(REcT);
    free(AiC); free(EcAi); free(RAi); free(AiEr); free(mem); free(lu);
    return st;
}

/* linalg::InvUpdate (linalg.cpp:402-573), ranks rc, rr in {0,1}; two rows
 * through inv_update_general. */
static int inv_update(const zc* A, zc* Ai, int N, const zc* C, const int* ci, int rc,
                      const zc* R, const int* ri, int rr, bigc* det, zc* work)
{
    if (!rc && !rr) { *det = bigc_make(1.0, 0); return ORC_OK; }
    if (rc <= 1 && rr == 2) return inv_update_general(A, Ai, N, C, ci, rc, R, ri, rr, det);
    if (rc > 1 || rr > 1) return ORC_ERR_INVALID;
    zc* AiC = work;            /* N */
    zc* RAi = work + N;        /* N */
    zc* AiEr = work + 2 * N;   /* N */
    zc* EcAi = work + 3 * N;   /* N */
    zc* mem = work + 4 * N;    /* N */
    zc* lu = work + 5 * N;     /* small */
    if (rc)
        for (int i = 0; i < N; ++i) {               /* zgemm N x 1 x N */
            zc s = 0.0;
            for (int l = 0; l < N; ++l) s += Ai[i + (size_t)l * N] * C[l];
            AiC[i] = s;
        }
    if (rr)
        for (int jj = 0; jj < N; ++jj) {            /* zgemm 1 x N x N */
            zc s = 0.0;
            for (int l = 0; l < N; ++l) s += R[l] * Ai[l + (size_t)jj * N];
            RAi[jj] = s;
        }
    zc EcAiC = rc ? AiC[ci[0]] : 0.0;
    zc RAiEr = rr ? RAi[ri[0]] : 0.0;
    zc RAiC = 0.0;
    if (rc && rr) for (int l = 0; l < N; ++l) RAiC += RAi[l] * C[l];
    zc ErTAEcT = 0.0, ErTC = 0.0, REcT = 0.0;
    if (rc && rr) { ErTAEcT = A[ri[0] + (size_t)ci[0] * N]; ErTC = C[ri[0]]; REcT = R[(size_t)ci[0]]; }
    int m = rc + rr;
    zc B[4] = {0, 0, 0, 0};
    if (rc && rr) B[m] = Ai[ci[0] + (size_t)ri[0] * N];   /* B12 */
    if (rr) B[rc + rc * m] = RAiEr;                       /* B22 */
    if (rc) B[0] = EcAiC;                                  /* B11 */
    if (rr && rc) { B[0] += -1.0 * B[2] * ErTC; B[0] += B[2] * ErTAEcT; }
    if (rr && rc) B[1] = RAiC - REcT;                      /* B21 */
    if (rr && rc) { B[1] += B[3] * ErTAEcT; B[1] += -1.0 * B[3] * ErTC; }
    zc Bi[4];
    if (det_inv(B, Bi, m, det, lu)) return ORC_ERR_SINGULAR;
    for (int i = 0; i < N; ++i) {
        if (rr) AiEr[i] = Ai[i + (size_t)ri[0] * N];
        if (rc) EcAi[i] = Ai[ci[0] + (size_t)i * N];
    }
    if (rr && rc)
        for (int i = 0; i < N; ++i) { AiC[i] += -1.0 * AiEr[i] * ErTC; AiC[i] += AiEr[i] * ErTAEcT; }
    if (rc) AiC[ci[0]] -= 1.0;
    if (rr) RAi[ri[0]] -= 1.0;
    if (rc) {
        for (int jj = 0; jj < N; ++jj) mem[jj] = Bi[0] * EcAi[jj];
        for (int jj = 0; jj < N; ++jj) { zc t = -mem[jj]; for (int i = 0; i < N; ++i) Ai[i + (size_t)jj * N] += t * AiC[i]; }
    }
    if (rc && rr) {
        for (int jj = 0; jj < N; ++jj) mem[jj] = Bi[m] * RAi[jj];          /* Bi12 */
        for (int jj = 0; jj < N; ++jj) { zc t = -mem[jj]; for (int i = 0; i < N; ++i) Ai[i + (size_t)jj * N] += t * AiC[i]; }
        for (int jj = 0; jj < N; ++jj) mem[jj] = Bi[1] * EcAi[jj];          /* Bi21 */
        for (int jj = 0; jj < N; ++jj) { zc t = -mem[jj]; for (int i = 0; i < N; ++i) Ai[i + (size_t)jj * N] += t * AiEr[i]; }
    }
    if (rr) {
        for (int jj = 0; jj < N; ++jj) mem[jj] = Bi[rc + rc * m] * RAi[jj];  /* Bi22 */
        for (int jj = 0; jj < N; ++jj) { zc t = -mem[jj]; for (int i = 0; i < N; ++i) Ai[i + (size_t)jj * N] += t * AiEr[i]; }
    }
    return ORC_OK;
}

/* SlaterDeterminant::Init (SlaterDeterminant.cpp:60-92) */
static int sd_init(orc_walker* w)
{
    orc_job* j = w->j;
    bigc d[2];
    for (int fl = 0; fl < 2; ++fl) {
        int N = j->N[fl];
        for (int r = 0; r < N; ++r)
            for (int f = 0; f < N; ++f)
                w->mat[fl][(size_t)r * N + f] = matel(j, w->wav.part[fl][f], w->lat.part[fl][r], fl);
    }
    for (int fl = 0; fl < 2; ++fl) det_inv(w->mat[fl], w->mati[fl], j->N[fl], &d[fl], w->work);
    int bad = 0;
    for (int fl = 0; fl < 2; ++fl) if (d[fl].e < -8 || bigc_is_zero(d[fl])) bad = 1;
    if (bad) { w->amp_ok = 0; w->amp = bigc_make(0.0, 0); }
    else { w->amp = d[0]; bigc_muleq(&w->amp, d[1]); w->amp_ok = 1; }
    return tl_err;
}

static bigc sd_amp(const orc_walker* w) { return bigc_mul_d(w->amp, (double)w->wav.sign); }  /* :94 */

/* SlaterDeterminant::VirtUpdate (SlaterDeterminant.cpp:96-268) */
static int sd_virt_update(const orc_walker* w, int Nr, const hopset* rh, int Nk, const hopset* kh, bigc* qs)
{
    const orc_job* j = w->j;
    if (!w->amp_ok) return ORC_ERR_ZERO_AMP;
    if (Nr * Nk == 0) return ORC_ERR_INVALID;
    int NN = Nr > Nk ? Nr : Nk;
    for (int nk = 0; nk < Nk; ++nk) {
        int sign = wav_hopsign(w, &kh[nk]);
        for (int nr = 0; nr < Nr; ++nr)
            qs[nk * Nr + nr] = bigc_mul_d(bigc_mul_d(w->amp, (double)w->wav.sign), (double)sign);
    }
    bigc* qq = (bigc*)malloc(sizeof(bigc) * NN);
    int rc_all = ORC_OK;
    for (int fl = 0; fl < 2 && !rc_all; ++fl) {
        int N = j->N[fl];
        int* ridx = (int*)malloc(sizeof(int) * Nr);
        int* kidx = (int*)malloc(sizeof(int) * Nk);
        ridx[0] = 0; kidx[0] = 0;
        for (int n = 1; n < Nr; ++n) ridx[n] = ridx[n - 1] + rh[n - 1].n[fl];
        for (int n = 1; n < Nk; ++n) kidx[n] = kidx[n - 1] + kh[n - 1].n[fl];
        int Nrf = ridx[Nr - 1] + rh[Nr - 1].n[fl];
        int Nkf = kidx[Nk - 1] + kh[Nk - 1].n[fl];
        zc* V = (zc*)malloc(sizeof(zc) * (size_t)N * (Nrf > 0 ? Nrf : 1));
        zc* U = (zc*)malloc(sizeof(zc) * (size_t)N * (Nkf > 0 ? Nkf : 1));
        for (int n = 0; n < Nr; ++n)
            if (rh[n].n[fl])
                for (int f = 0; f < N; ++f)
                    V[(size_t)ridx[n] * N + f] = matel(j, w->wav.part[fl][f], rh[n].to[fl], fl);
        for (int n = 0; n < Nk; ++n)
            for (int r = 0; r < kh[n].n[fl]; ++r)
                for (int f = 0; f < N; ++f)
                    U[(size_t)f * Nkf + kidx[n] + r] = matel(j, hop_to(&kh[n], fl, r), w->lat.part[fl][f], fl);
        int* rfid = (int*)malloc(sizeof(int) * (Nrf > 0 ? Nrf : 1));
        int* kfid = (int*)malloc(sizeof(int) * (Nkf > 0 ? Nkf : 1));
        int* rfr = (int*)malloc(sizeof(int) * Nr);
        int* kfr = (int*)malloc(sizeof(int) * Nk);
        for (int nr = 0; nr < Nr; ++nr) {
            rfr[nr] = rh[nr].n[fl];
            if (rh[nr].n[fl]) rfid[ridx[nr]] = w->lat.fock[fl][rh[nr].from[fl]];
        }
        for (int nk = 0; nk < Nk; ++nk) {
            kfr[nk] = kh[nk].n[fl];
            for (int rk = 0; rk < kh[nk].n[fl]; ++rk) kfid[kidx[nk] + rk] = w->wav.fock[fl][hop_from(&kh[nk], fl, rk)];
        }
        if (Nk == NN) {
            for (int nr = 0; nr < Nr && !rc_all; ++nr) {
                if (rh[nr].n[fl])
                    for (int nk = 0; nk < Nk; ++nk)
                        for (int rk = 0; rk < kh[nk].n[fl]; ++rk)
                            U[(size_t)rfid[ridx[nr]] * Nkf + kidx[nk] + rk] =
                                matel(j, hop_to(&kh[nk], fl, rk), rh[nr].to[fl], fl);
                rc_all = det_update(w->mat[fl], w->mati[fl], N, &V[(size_t)ridx[nr] * N], N,
                                    &rfid[ridx[nr]], &rfr[nr], 1, U, Nkf, kfid, kfr, Nk, qq, w->work);
                for (int nk = 0; nk < Nk; ++nk) bigc_muleq(&qs[nk * Nr + nr], qq[nk]);
                if (rh[nr].n[fl])
                    for (int nk = 0; nk < Nk; ++nk)
                        for (int rk = 0; rk < kh[nk].n[fl]; ++rk)
                            U[(size_t)rfid[ridx[nr]] * Nkf + kidx[nk] + rk] =
                                matel(j, hop_to(&kh[nk], fl, rk), w->lat.part[fl][rfid[ridx[nr]]], fl);
            }
        } else {
            for (int nk = 0; nk < Nk && !rc_all; ++nk) {
                for (int rk = 0; rk < kh[nk].n[fl]; ++rk)
                    for (int nr = 0; nr < Nr; ++nr)
                        if (rh[nr].n[fl])
                            V[(size_t)ridx[nr] * N + kfid[kidx[nk] + rk]] =
                                matel(j, hop_to(&kh[nk], fl, rk), rh[nr].to[fl], fl);
                rc_all = det_update(w->mat[fl], w->mati[fl], N, V, N, rfid, rfr, Nr,
                                    &U[kidx[nk]], Nkf, &kfid[kidx[nk]], &kfr[nk], 1, qq, w->work);
                for (int nr = 0; nr < Nr; ++nr) bigc_muleq(&qs[nk * Nr + nr], qq[nr]);
                for (int rk = 0; rk < kh[nk].n[fl]; ++rk)
                    for (int nr = 0; nr < Nr; ++nr)
                        if (rh[nr].n[fl])
                            V[(size_t)ridx[nr] * N + kfid[kidx[nk] + rk]] =
                                matel(j, w->wav.part[fl][kfid[kidx[nk] + rk]], rh[nr].to[fl], fl);
            }
        }
        free(V); free(U); free(rfid); free(kfid); free(rfr); free(kfr); free(ridx); free(kidx);
    }
    free(qq);
    if (!rc_all && tl_err) rc_all = tl_err;
    return rc_all;
}

/* SlaterDeterminant::Update (SlaterDeterminant.cpp:270-326) */
static int sd_update(orc_walker* w, const hopset* rh, const hopset* kh)
{
    orc_job* j = w->j;
    if (!w->amp_ok) return ORC_ERR_ZERO_AMP;
    for (int fl = 0; fl < 2; ++fl) {
        int N = j->N[fl];
        zc* V = w->work + 8 * (size_t)N + 16;
        zc* U = V + N;   /* kh->n[fl] rows, U[f * n + r] */
        const int nk = kh->n[fl];
        int rid = 0, kid[2] = {0, 0};
        if (rh->n[fl])
            for (int f = 0; f < N; ++f) V[f] = matel(j, w->wav.part[fl][f], rh->to[fl], fl);
        for (int r = 0; r < nk; ++r)
            for (int f = 0; f < N; ++f) U[(size_t)f * nk + r] = matel(j, hop_to(kh, fl, r), w->lat.part[fl][f], fl);
        for (int r = 0; r < nk; ++r) kid[r] = w->wav.fock[fl][hop_to(kh, fl, r)];
        if (rh->n[fl]) rid = w->lat.fock[fl][rh->to[fl]];
        bigc qq;
        int rc = inv_update(w->mat[fl], w->mati[fl], N, V, &rid, rh->n[fl], U, kid, nk, &qq, w->work);
        if (rc) return rc;
        bigc_muleq(&w->amp, qq);
    }
    return tl_err;
}

/* LatticeStepper::weight (LatticeStepper.cpp:149-169), non-const version */
static int ls_weight(orc_walker* w)
{
    if (bigd_d(w->weight) < 0.0) {
        int Nk = w->j->Nexc;
        hopset e = hopset_empty();
        bigc* qs = (bigc*)malloc(sizeof(bigc) * Nk);
        int rc = sd_virt_update(w, 1, &e, Nk, wav_gethops(w), qs);
        bigd out = bigd_make(0.0, 0);
        for (int k = 0; k < Nk; ++k) bigd_addeq(&out, bigc_norm(qs[k]));
        free(qs);
        w->weight = out;
        return rc;
    }
    return ORC_OK;
}

/* LatticeStepper::trystep (LatticeStepper.cpp:36-100) */
static int ls_trystep(orc_walker* w, bigd* out, orc_trace* tr)
{
    orc_job* j = w->j;
    double u1 = rng_uniform(&w->rng);
    int v1 = (int)((double)j->Ns * u1);
    double u2 = rng_uniform(&w->rng);
    int v2 = j->nbr[v1 * 4 + (int)((double)j->deg[v1] * u2)];
    /* GetLatOc: occupied flavour at the vertex (max_element by size, first wins) */
    int f1 = (w->lat.fock[0][v1] != w->lat.Npt[0]) ? 0 : ((w->lat.fock[1][v1] != w->lat.Npt[1]) ? 1 : 0);
    int f2 = (w->lat.fock[0][v2] != w->lat.Npt[0]) ? 0 : ((w->lat.fock[1][v2] != w->lat.Npt[1]) ? 1 : 0);
    double u3 = rng_uniform(&w->rng);
    (void)u3;
    if (tr) { tr->v1 = v1; tr->v2 = v2; tr->u[0] = u1; tr->u[1] = u2; tr->u[2] = u3; }
    w->prev = hopset_empty();
    if (f1 == f2) {
        w->khop = -1;
        w->prev_weight = w->weight;
        *out = w->weight;
        if (tr) tr->kind = 0;
        return ORC_OK;
    }
    w->prev.n[f1] = 1; w->prev.from[f1] = v1; w->prev.to[f1] = v2;
    w->prev.n[f2] = 1; w->prev.from[f2] = v2; w->prev.to[f2] = v1;
    if (tr) tr->kind = 1;
    int Nk = j->Nexc;
    bigc* qs = (bigc*)malloc(sizeof(bigc) * Nk);
    int rc = sd_virt_update(w, 1, &w->prev, Nk, wav_gethops(w), qs);
    bigd s = bigd_make(0.0, 0);
    for (int k = 0; k < Nk; ++k) bigd_addeq(&s, bigc_norm(qs[k]));
    int best = 0;
    for (int k = 1; k < Nk; ++k)
        if (bigd_lt(bigc_norm(qs[best]), bigc_norm(qs[k]))) best = k;
    free(qs);
    w->khop = best;
    w->prev_weight = s;
    *out = s;
    return rc;
}

/* LatticeStepper::step (LatticeStepper.cpp:102-147) */
static int ls_step(orc_walker* w)
{
    state_hop(&w->lat, &w->prev);
    int rc;
    if (w->khop >= 0) {
        hopset kh = wav_gethops(w)[w->khop];
        wav_hop(w, w->khop);
        rc = sd_update(w, &w->prev, &kh);
    } else {
        hopset e = hopset_empty();
        rc = sd_update(w, &w->prev, &e);
    }
    if (rc) return rc;
    if (bigc_is_zero(sd_amp(w))) return ORC_ERR_ZERO_AMP;
    w->weight = bigd_make(-1.0, 0);
    rc = ls_weight(w);
    if (rc) return rc;
    if (bigd_d(w->prev_weight) >= 0.0 &&
        fabs(bigd_d(bigd_div(w->prev_weight, w->weight)) - 1) > 1e-6)
        return ORC_ERR_WEIGHT;
    w->prev = hopset_empty();
    w->khop = -1;
    return ORC_OK;
}

/* MetroMC::YesNo (MetroMC.cpp:27-43) */
static int mc_yesno(orc_walker* w, bigd in, double* u4)
{
    double din = bigd_d(in);
    double u = rng_uniform(&w->rng);
    *u4 = u;
    return din > 1.0 ? u < 1 : u < din;
}

/* MetroMC::Step (MetroMC.cpp:90-103) */
int orc_walker_step(orc_walker* w, int meas, orc_trace* tr)
{
    tl_err = 0;
    bigd nw;
    if (tr) memset(tr, 0, sizeof *tr);
    int rc = ls_trystep(w, &nw, tr);
    if (rc) return rc;
    bigd ratio = bigd_div(nw, w->state_weight);
    double u4;
    int acc = mc_yesno(w, ratio, &u4);
    if (tr) {
        tr->u[3] = u4; tr->ratio = bigd_d(ratio); tr->accepted = acc;
        tr->w_new_c = nw.c; tr->w_new_e = nw.e; tr->khop = w->khop;
    }
    int real = w->prev.n[0] || w->prev.n[1];
    if (acc) {
        rc = ls_step(w);
        if (rc) return rc;
        w->state_weight = nw;
        if (real) { w->accepted_real++; w->since_reinv++; }
    } else if (meas) w->rejection++;
    if (meas) w->steps++;
    return tl_err;
}

/* ------------------------------------------------------------------ */
/* ProjHeis::measure (ProjHeis.cpp:40-158), Bx = 0, J = 1 on every edge. */
static int q_projheis(orc_walker* w)
{
    orc_job* j = w->j;
    int Nexc = j->Nexc;
    bigd weight = w->weight;   /* m_stepper->weight() const */
    int nsw = 0;
    hopset* rh = (hopset*)malloc(sizeof(hopset) * (j->nedge + 1));
    for (int e = 0; e < j->nedge; ++e) {
        int vi = j->edge_i[e], vj = j->edge_j[e];
        int fi = (w->lat.fock[0][vi] != w->lat.Npt[0]) ? 0 : 1;
        int fj = (w->lat.fock[0][vj] != w->lat.Npt[0]) ? 0 : 1;
        if (fi != fj) {
            hopset h = hopset_empty();
            h.n[fi] = 1; h.from[fi] = vi; h.to[fi] = vj;
            h.n[fj] = 1; h.from[fj] = vj; h.to[fj] = vi;
            rh[nsw++] = h;
        }
    }
    rh[nsw++] = hopset_empty();
    bigc* qs = (bigc*)malloc(sizeof(bigc) * (size_t)nsw * Nexc);
    int rc = sd_virt_update(w, nsw, rh, Nexc, wav_gethops(w), qs);
    if (rc) { free(rh); free(qs); return rc; }
    bigc* amps = (bigc*)malloc(sizeof(bigc) * Nexc);
    bigc* heis = (bigc*)malloc(sizeof(bigc) * Nexc);
    for (int k = 0; k < Nexc; ++k) { amps[k] = qs[(size_t)k * nsw + nsw - 1]; heis[k] = bigc_make(0.0, 0); }
    int swc = 0;
    for (int e = 0; e < j->nedge; ++e) {
        double J = 1.0;
        int vi = j->edge_i[e], vj = j->edge_j[e];
        int fi = (w->lat.fock[0][vi] != w->lat.Npt[0]) ? 0 : 1;
        int fj = (w->lat.fock[0][vj] != w->lat.Npt[0]) ? 0 : 1;
        if (fi != fj) {
            for (int k = 0; k < Nexc; ++k) {
                bigc t = bigc_add(bigc_mul_d(amps[k], 0.25), bigc_mul_d(qs[(size_t)k * nsw + swc], 0.5));
                bigc_subeq(&heis[k], bigc_mul_d(t, J));
            }
            ++swc;
        } else {
            for (int k = 0; k < Nexc; ++k) bigc_addeq(&heis[k], bigc_mul_d(amps[k], J * 0.25));
        }
    }
    if (Nexc == 1) {
        bigc v = bigc_div_d(bigc_div_d(bigc_div_bd(bigc_mul(heis[0], bigc_conj(amps[0])), weight), (double)j->L), (double)j->L);
        w->pj_vals[0] += bigc_z(v);
        w->pj_vals[1] += 1;
    } else {
        for (int k1 = 0; k1 < Nexc; ++k1)
            for (int k2 = 0; k2 < Nexc; ++k2) {
                w->pj_vals[(size_t)k1 * Nexc + k2] += bigc_z(bigc_div_bd(bigc_mul(bigc_conj(amps[k1]), heis[k2]), weight));
                w->pj_vals[(size_t)(Nexc + k1) * Nexc + k2] +=
                    bigc_z(bigc_div_bd(bigc_mul(bigc_conj(amps[k1]), amps[k2]), weight));
            }
    }
    free(rh); free(qs); free(amps); free(heis);
    return tl_err;
}

/* StagMagnZ::measure (StagMagnZ.cpp:12-43) */
static void q_stagmagn(orc_walker* w)
{
    orc_job* j = w->j;
    zc msz = 0.0;
    for (int v = 0; v < j->Ns; ++v) {
        int x = v % j->L, y = v / j->L;
        zc ph = cexp(cplx(0.0, M_PI * (double)(x + y)));
        int up = (w->lat.fock[0][v] != w->lat.Npt[0]) ? 1 : 0;
        msz += ph * (double)(2 * up - 1);
    }
    msz /= (double)j->Ns;
    w->sm_val += msz;
}

/* StatSpinStruct::measure (StatSpinStruct.cpp:16-135), two flavours. */
static int q_statspin(orc_walker* w)
{
    orc_job* j = w->j;
    int N = j->Ns;
    size_t nh = 0;
    hopset* hops = (hopset*)malloc(sizeof(hopset) * ((size_t)N * (N + 1) / 2 + 1));
    for (int vi = 0; vi < N; ++vi)
        for (int vj = vi; vj < N; ++vj) {
            int fi = (w->lat.fock[0][vi] != w->lat.Npt[0]) ? 0 : 1;
            int fj = (w->lat.fock[0][vj] != w->lat.Npt[0]) ? 0 : 1;
            if (fi != fj) {
                hopset h = hopset_empty();
                h.n[fi] = 1; h.from[fi] = vi; h.to[fi] = vj;
                h.n[fj] = 1; h.from[fj] = vj; h.to[fj] = vi;
                hops[nh++] = h;
            }
        }
    bigc amp = sd_amp(w);
    bigc* sw = (bigc*)malloc(sizeof(bigc) * (nh ? nh : 1));
    int rc = ORC_OK;
    if (nh) {
        hopset e = hopset_empty();
        rc = sd_virt_update(w, (int)nh, hops, 1, &e, sw);
    }
    if (rc) { free(hops); free(sw); return rc; }
    zc* szz = &w->ss_vals[0];
    zc* spm = &w->ss_vals[(size_t)N * N];
    zc* smp = &w->ss_vals[2 * (size_t)N * N];
    bigd wt = w->weight;
    size_t s = 0;
    bigc ca = bigc_conj(amp);
    for (int vi = 0; vi < N; ++vi)
        for (int vj = vi; vj < N; ++vj) {
            int upi = (w->lat.fock[0][vi] != w->lat.Npt[0]);
            int upj = (w->lat.fock[0][vj] != w->lat.Npt[0]);
            size_t ij = (size_t)vi * N + vj, ji = (size_t)vj * N + vi;
            if (upi) {
                if (upj) {
                    if (vi == vj) { spm[ij] += 1.0; szz[ij] += 0.25; }
                    else { szz[ij] += 0.25; szz[ji] += 0.25; }
                } else {
                    szz[ij] += -0.25; szz[ji] += -0.25;
                    zc v = bigc_z(bigc_div_bd(bigc_mul(ca, sw[s]), wt));
                    smp[ij] += -v; spm[ji] += -v;
                    ++s;
                }
            } else {
                if (upj) {
                    szz[ij] += -0.25; szz[ji] += -0.25;
                    zc v = bigc_z(bigc_div_bd(bigc_mul(ca, sw[s]), wt));
                    spm[ij] += -v; smp[ji] += -v;
                    ++s;
                } else {
                    if (vi == vj) { smp[ij] += 1.0; szz[ij] += 0.25; }
                    else { szz[ij] += 0.25; szz[ji] += 0.25; }
                }
            }
        }
    free(hops); free(sw);
    return tl_err;
}

int orc_walker_measure(orc_walker* w, int mask)
{
    tl_err = 0;
    int rc = ORC_OK;
    if (mask & ORC_MEAS_PROJHEIS) { rc = q_projheis(w); if (rc) return rc; w->meas_pj++; }
    if (mask & ORC_MEAS_STAGMAGN) { q_stagmagn(w); w->meas_sm++; }
    if (mask & ORC_MEAS_STATSPIN) { rc = q_statspin(w); if (rc) return rc; w->meas_ss++; }
    return tl_err;
}

void orc_walker_reset_quantities(orc_walker* w)   /* Quantity::init and derived */
{
    int Nexc = w->j->Nexc, Ns = w->j->Ns;
    memset(w->pj_vals, 0, sizeof(zc) * 2 * (size_t)Nexc * Nexc);
    w->sm_val = 0.0;
    memset(w->ss_vals, 0, sizeof(zc) * 5 * (size_t)Ns * Ns);
    w->meas_pj = w->meas_sm = w->meas_ss = 0;
}

int orc_walker_reinit(orc_walker* w)
{
    tl_err = 0;
    int rc = sd_init(w);
    w->reinversions++;
    w->since_reinv = 0;
    if (!w->amp_ok) return ORC_ERR_SINGULAR;
    return rc;
}

/* MetroMC::Walk (MetroMC.cpp:45-88) */
int orc_walker_walk(orc_walker* w, uint64_t len, uint64_t meas, int mask, int reinv_every, orc_trace* traces)
{
    if (meas) orc_walker_reset_quantities(w);
    for (uint64_t s = 0; s < len; ++s) {
        int rc = orc_walker_step(w, meas != 0, traces ? &traces[s] : NULL);
        if (rc) return rc;
        if (reinv_every > 0 && w->since_reinv >= (uint64_t)reinv_every) {
            rc = orc_walker_reinit(w);
            if (rc) return rc;
        }
        if (meas && (meas == 1 || s % meas == 0)) {
            rc = orc_walker_measure(w, mask);
            if (rc) return rc;
        }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
orc_walker* orc_walker_create(orc_job* j, uint64_t seed, uint32_t walker_id)
{
    orc_walker* w = (orc_walker*)calloc(1, sizeof(orc_walker));
    w->j = j;
    state_init(&w->lat, j->N, (int[2]){j->Ns, j->Ns});
    state_copy(&w->wav, &j->wav0);
    w->cur = 0;
    int Nmax = j->N[0] > j->N[1] ? j->N[0] : j->N[1];
    for (int fl = 0; fl < 2; ++fl) {
        w->mat[fl] = (zc*)calloc((size_t)j->N[fl] * j->N[fl] + 1, sizeof(zc));
        w->mati[fl] = (zc*)calloc((size_t)j->N[fl] * j->N[fl] + 1, sizeof(zc));
    }
    w->work = (zc*)calloc(16 * (size_t)Nmax + 64 + (size_t)j->Ns, sizeof(zc));
    w->amp = bigc_make(0.0, 0);
    w->amp_ok = 0;
    w->prev = hopset_empty();
    w->khop = -1;
    w->weight = bigd_make(-1.0, 0);
    w->prev_weight = bigd_make(-1.0, 0);
    w->state_weight = bigd_make(-1.0, 0);
    w->rng.seed = seed; w->rng.walker = walker_id; w->rng.stream = 0; w->rng.next = 0;
    w->pj_vals = (zc*)calloc(2 * (size_t)j->Nexc * j->Nexc, sizeof(zc));
    w->ss_vals = (zc*)calloc(5 * (size_t)j->Ns * j->Ns, sizeof(zc));
    return w;
}

void orc_walker_destroy(orc_walker* w)
{
    if (!w) return;
    state_free(&w->lat); state_free(&w->wav);
    for (int fl = 0; fl < 2; ++fl) { free(w->mat[fl]); free(w->mati[fl]); }
    free(w->work); free(w->pj_vals); free(w->ss_vals);
    free(w);
}

/* vmc.cpp:243-263: pick the channel state of largest overlap, build the
 * stepper (weight cached by the MetroMC constructor, MetroMC.cpp:24). */
static int start_finish(orc_walker* w)
{
    orc_job* j = w->j;
    bigd maxq = bigc_norm(sd_amp(w));
    int kmax = w->cur;
    for (int k = 0; k < j->Nexc; ++k) {
        wav_hop(w, k);
        sd_init(w);
        bigd n = bigc_norm(sd_amp(w));
        if (bigd_gt(n, maxq)) { kmax = k; maxq = n; }
    }
    wav_hop(w, kmax);
    sd_init(w);
    if (!w->amp_ok) return ORC_ERR_SINGULAR;
    w->prev = hopset_empty();
    w->khop = -1;
    w->weight = bigd_make(-1.0, 0);
    w->prev_weight = bigd_make(-1.0, 0);
    int rc = ls_weight(w);
    w->state_weight = w->weight;
    return rc ? rc : tl_err;
}

int orc_walker_set_config(orc_walker* w, const int8_t* up)
{
    tl_err = 0;
    orc_job* j = w->j;
    int cnt = 0;
    for (int v = 0; v < j->Ns; ++v) cnt += up[v] ? 1 : 0;
    if (cnt != j->N[0]) return ORC_ERR_INVALID;
    /* LatticeState::FockInit (LatticeState.cpp:84-113) */
    int* st[2];
    for (int fl = 0; fl < 2; ++fl) {
        st[fl] = (int*)malloc(sizeof(int) * j->Ns);
        for (int v = 0; v < j->Ns; ++v) {
            int occ = fl == 0 ? (up[v] != 0) : (up[v] == 0);
            st[fl][v] = occ ? 0 : j->N[fl];
        }
    }
    state_initfock(&w->lat, st);
    free(st[0]); free(st[1]);
    sd_init(w);
    return start_finish(w);
}

int orc_walker_random_start(orc_walker* w)
{
    tl_err = 0;
    orc_job* j = w->j;
    rng_t r = w->rng;
    r.stream = 1; r.next = 0;
    int tc = 0, failcount = 10;
    int* fst[2];
    fst[0] = (int*)malloc(sizeof(int) * j->Ns);
    fst[1] = (int*)malloc(sizeof(int) * j->Ns);
    while (bigc_is_zero(sd_amp(w)) && tc < failcount) {
        /* LatticeState::RanInit (LatticeState.cpp:37-82) */
        for (int fl = 0; fl < 2; ++fl) for (int v = 0; v < j->Ns; ++v) fst[fl][v] = j->N[fl];
        for (int fl = 0; fl < 2; ++fl) {
            int np = 0;
            int NTpt = j->N[0] + j->N[1];
            if (fl == 1 && NTpt == j->Ns) {
                for (int v = 0; v < j->Ns; ++v) {
                    int occ = (fst[0][v] < j->N[0]) || (fst[1][v] < j->N[1]);
                    if (!occ) fst[fl][v] = np++;
                }
            } else {
                while (np != j->N[fl]) {
                    int v = (int)(rng_uniform(&r) * (double)j->Ns);
                    int occ = (fst[0][v] < j->N[0]) || (fst[1][v] < j->N[1]);
                    if (!occ) fst[fl][v] = np++;
                }
            }
        }
        state_initfock(&w->lat, fst);
        sd_init(w);
        tc++;
    }
    free(fst[0]); free(fst[1]);
    if (tc == failcount) return ORC_ERR_SINGULAR;
    return start_finish(w);
}

void orc_walker_rng_seek(orc_walker* w, uint64_t k) { w->rng.stream = 0; w->rng.next = k; }

void orc_walker_config(const orc_walker* w, int8_t* up)
{
    for (int v = 0; v < w->j->Ns; ++v) up[v] = (int8_t)(w->lat.fock[0][v] != w->lat.Npt[0]);
}

void orc_walker_particles(const orc_walker* w, int fl, int32_t* part)
{
    for (int p = 0; p < w->j->N[fl]; ++p) part[p] = w->lat.part[fl][p];
}

void orc_walker_amp(const orc_walker* w, double* mant, int32_t* e)
{
    bigc a = sd_amp(w);
    mant[0] = creal(a.c); mant[1] = cimag(a.c); *e = a.e;
}

void orc_walker_weight(const orc_walker* w, double* mant, int32_t* e) { *mant = w->weight.c; *e = w->weight.e; }

void orc_walker_inverse(const orc_walker* w, int fl, double* out)
{
    size_t n = (size_t)w->j->N[fl] * w->j->N[fl];
    for (size_t i = 0; i < n; ++i) { out[2 * i] = creal(w->mati[fl][i]); out[2 * i + 1] = cimag(w->mati[fl][i]); }
}

int orc_walker_current_state(const orc_walker* w) { return w->cur; }

void orc_walker_counts(const orc_walker* w, uint64_t* steps, uint64_t* rej, uint64_t* acc, uint64_t* reinv)
{
    if (steps) *steps = w->steps;
    if (rej) *rej = w->rejection;
    if (acc) *acc = w->accepted_real;
    if (reinv) *reinv = w->reinversions;
}

int orc_walker_projheis(const orc_walker* w, double* vals)
{
    size_t n = 2 * (size_t)w->j->Nexc * w->j->Nexc;
    for (size_t i = 0; i < n; ++i) { vals[2 * i] = creal(w->pj_vals[i]); vals[2 * i + 1] = cimag(w->pj_vals[i]); }
    return w->meas_pj;
}

int orc_walker_stagmagn(const orc_walker* w, double* val)
{
    val[0] = creal(w->sm_val); val[1] = cimag(w->sm_val);
    return w->meas_sm;
}

int orc_walker_statspin(const orc_walker* w, double* vals)
{
    size_t n = 5 * (size_t)w->j->Ns * w->j->Ns;
    for (size_t i = 0; i < n; ++i) { vals[2 * i] = creal(w->ss_vals[i]); vals[2 * i + 1] = cimag(w->ss_vals[i]); }
    return w->meas_ss;
}

int orc_walker_virt_update(const orc_walker* w, int nset, const int32_t* hops, double* out)
{
    tl_err = 0;
    hopset* rh = (hopset*)malloc(sizeof(hopset) * (nset > 0 ? nset : 1));
    for (int i = 0; i < nset; ++i) {
        rh[i] = hopset_empty();
        for (int fl = 0; fl < 2; ++fl)
            if (hops[4 * i + 2 * fl] >= 0) {
                rh[i].n[fl] = 1; rh[i].from[fl] = hops[4 * i + 2 * fl]; rh[i].to[fl] = hops[4 * i + 2 * fl + 1];
            }
    }
    int Nk = w->j->Nexc;
    bigc* qs = (bigc*)malloc(sizeof(bigc) * (size_t)nset * Nk);
    int rc = sd_virt_update(w, nset, rh, Nk, wav_gethops(w), qs);
    for (size_t i = 0; i < (size_t)nset * Nk; ++i) {
        out[3 * i] = creal(qs[i].c); out[3 * i + 1] = cimag(qs[i].c); out[3 * i + 2] = qs[i].e;
    }
    free(rh); free(qs);
    return rc;
}
