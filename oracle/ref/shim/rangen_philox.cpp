// Link-time replacement for the reference's RanGen.cpp (same RanGen.h
// interface) used only by the parity oracle (oracle/_ref).  uniform() draws
// the Philox4x32-10 stream that the GPU engine draws: counter
// {call_lo, call_hi, walker, stream}, key {seed_lo, seed_hi}, two uniforms
// per call, u = (52-bit integer + 1/2) * 2^-52 in (0,1).
#include "RanGen.h"
#include <cstdint>

struct state_t {
    uint64_t seed;
    uint32_t walker, stream;
    uint64_t next;
};

static state_t g_state = {0, 0, 0, 0};

static void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1; c3 = (uint32_t)p0; c0 = n0; c2 = n2;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double draw(state_t* s)
{
    uint64_t k = s->next++;
    uint64_t call = k >> 1;
    uint32_t ctr[4] = {(uint32_t)call, (uint32_t)(call >> 32), s->walker, s->stream};
    uint32_t key[2] = {(uint32_t)s->seed, (uint32_t)(s->seed >> 32)};
    uint32_t x[4];
    philox4x32_10(ctr, key, x);
    uint32_t a = (k & 1) ? x[2] : x[0], b = (k & 1) ? x[3] : x[1];
    uint64_t m = (((uint64_t)a << 20) ^ (uint64_t)(b >> 12)) & ((((uint64_t)1) << 52) - 1);
    return ((double)m + 0.5) * (1.0 / 4503599627370496.0);
}

RanGen::RanGen() { m_rng = &g_state; }
RanGen::~RanGen() {}
void RanGen::srand(size_t seed) { g_state.seed = seed; g_state.next = 0; }
double RanGen::uniform() { return draw(&g_state); }
RanGen RanGen::m_ran;

extern "C" void ref_rng_set(uint64_t seed, uint32_t walker, uint32_t stream, uint64_t next)
{
    g_state.seed = seed; g_state.walker = walker; g_state.stream = stream; g_state.next = next;
}
extern "C" uint64_t ref_rng_next(void) { return g_state.next; }
extern "C" double ref_rng_peek(uint64_t k)
{
    state_t s = g_state;
    s.next = k;
    return draw(&s);
}
