/*
 * orc_rng.c : Philox4x32-10 counter stream and CUDA texture-filter emulation for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Philox4x32-10 is written from the Random123 paper (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
 * as easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies with the published multipliers and
 * Weyl key increments.  The stream layout is the one the reference obtains from curand_init(seed,
 * subsequence, offset) followed by skipahead(skipahead_event_offset*event) (qudarap/qrng.h:131-137):
 * the 128-bit counter holds (draw/4 in the low 64 bits, subsequence in the high 64 bits), the key is the
 * 64-bit seed, each counter value yields four 32-bit outputs used in order, and a 32-bit output x maps to
 * the float uniform x*2^-32 + 2^-33 in (0,1].  Equality with curand's own host implementation is checked
 * by tests/test_oracle_rng.py against the reference build in oracle/_ref.
 *
 * The texture emulation follows the CUDA C Programming Guide appendix "Texture Fetching", linear
 * filtering: texel coordinate xB = x*N - 0.5, i = floor(xB), alpha = frac(xB) held with 8 fractional
 * bits, result = (1-alpha) T[i] + alpha T[i+1], bilinear in 2D; wrap addressing takes indices modulo N.
 * The reference creates both its textures with linear filtering, normalized coordinates and wrap
 * addressing (qudarap/QTex.cc:260-272, QBnd.cc:157-161, QScint.cc:104-109).
 */
#include <string.h>
#include "orc_internal.h"

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

static void philox10(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void ctr_add_lo(uint32_t c[4], uint64_t n)
{
    uint64_t lo = ((uint64_t)c[1] << 32 | c[0]);
    uint64_t nlo = lo + n;
    uint64_t carry = nlo < lo ? 1u : 0u;
    c[0] = (uint32_t)nlo; c[1] = (uint32_t)(nlo >> 32);
    if (carry) {
        uint64_t hi = ((uint64_t)c[3] << 32 | c[2]) + 1u;
        c[2] = (uint32_t)hi; c[3] = (uint32_t)(hi >> 32);
    }
}

static void ctr_add_hi(uint32_t c[4], uint64_t n)
{
    uint64_t hi = ((uint64_t)c[3] << 32 | c[2]) + n;
    c[2] = (uint32_t)hi; c[3] = (uint32_t)(hi >> 32);
}

void orc_rng_skipahead(orc_rng* r, uint64_t n)
{
    int lane = r->lane + (int)(n & 3u);
    uint64_t blocks = n >> 2;
    if (lane > 3) { blocks += 1; lane -= 4; }
    r->lane = lane;
    ctr_add_lo(r->ctr, blocks);
    philox10(r->ctr, r->key, r->out);
}

void orc_rng_init(orc_rng* r, uint64_t seed, uint64_t subsequence, uint64_t offset)
{
    memset(r, 0, sizeof(*r));
    r->key[0] = (uint32_t)seed;
    r->key[1] = (uint32_t)(seed >> 32);
    ctr_add_hi(r->ctr, subsequence);
    orc_rng_skipahead(r, offset);
}

float orc_uniform(orc_rng* r)
{
    uint32_t x = r->out[r->lane];
    r->lane += 1;
    if (r->lane == 4) {
        ctr_add_lo(r->ctr, 1u);
        philox10(r->ctr, r->key, r->out);
        r->lane = 0;
    }
    const float two_m32 = 2.3283064365386963e-10f;   /* 2^-32 */
    return (float)x * two_m32 + two_m32 / 2.0f;
}

void orc_philox_uniforms(uint64_t seed, uint64_t subsequence, uint64_t offset, uint64_t skip, int n, float* out)
{
    orc_rng r;
    orc_rng_init(&r, seed, subsequence, offset);
    if (skip) orc_rng_skipahead(&r, skip);
    for (int i = 0; i < n; i++) out[i] = orc_uniform(&r);
}

/* ---- texture filtering ----------------------------------------------------------------------
 *
 * Precision details that the Programming Guide leaves open were measured on GB300 texture units through the
 * engine's own lookup kernel (tests/test_gpu_parity.py checks them on every GPU run):
 *   - the wrapped normalized coordinate is truncated to 21 fractional bits before scaling by N;
 *   - the 8-bit weight rounds half up;
 *   - the weighted sum is formed exactly and rounded once to binary32, ties away from zero.
 */

static inline void texel_coord(float x, int n, int* i0, int* i1, double* w)
{
    double xs = (double)x - floor((double)x);                   /* wrap */
    double xq = floor(xs * 2097152.0) / 2097152.0;              /* 21 fractional bits */
    double u = xq * (double)n - 0.5;
    double fi = floor(u);
    *w = floor((u - fi) * 256.0 + 0.5) / 256.0;                 /* 8-bit weight, half up */
    long i = (long)fi;
    i = ((i % n) + n) % n;
    *i0 = (int)i;
    *i1 = (int)((i + 1) % n);
}

static inline float round_ties_away(double e)
{
    float f = (float)e;
    double back = (double)f;
    if (back == e) return f;
    float other = back < e ? nextafterf(f, INFINITY) : nextafterf(f, -INFINITY);
    if (fabs((double)other - e) == fabs(back - e) && fabsf(other) > fabsf(f)) return other;
    return f;
}

static inline float blend(double a, double b, float T00, float T10, float T01, float T11)
{
    double e = (1.0 - a) * (1.0 - b) * (double)T00 + a * (1.0 - b) * (double)T10 +
               (1.0 - a) * b * (double)T01 + a * b * (double)T11;
    return round_ties_away(e);
}

v4 orc_tex2d4(const orc_tex* t, float x, float y)
{
    int x0, x1, y0, y1;
    double a, b;
    texel_coord(x, t->nx, &x0, &x1, &a);
    texel_coord(y, t->ny, &y0, &y1, &b);
    const float* T00 = t->data + 4 * ((size_t)y0 * t->nx + x0);
    const float* T10 = t->data + 4 * ((size_t)y0 * t->nx + x1);
    const float* T01 = t->data + 4 * ((size_t)y1 * t->nx + x0);
    const float* T11 = t->data + 4 * ((size_t)y1 * t->nx + x1);
    float r[4];
    for (int k = 0; k < 4; k++) r[k] = blend(a, b, T00[k], T10[k], T01[k], T11[k]);
    return V4(r[0], r[1], r[2], r[3]);
}

float orc_tex2d1(const orc_tex* t, float x, float y)
{
    int x0, x1, y0, y1;
    double a, b;
    texel_coord(x, t->nx, &x0, &x1, &a);
    texel_coord(y, t->ny, &y0, &y1, &b);
    return blend(a, b, t->data[(size_t)y0 * t->nx + x0], t->data[(size_t)y0 * t->nx + x1],
                 t->data[(size_t)y1 * t->nx + x0], t->data[(size_t)y1 * t->nx + x1]);
}

void orc_tex_lookup4(const orc_tex* t, const float* xy, int n, float* out)
{
    for (int i = 0; i < n; i++) {
        v4 v = orc_tex2d4(t, xy[2 * i], xy[2 * i + 1]);
        out[4 * i + 0] = v.x; out[4 * i + 1] = v.y; out[4 * i + 2] = v.z; out[4 * i + 3] = v.w;
    }
}

void orc_tex_lookup1(const orc_tex* t, const float* xy, int n, float* out)
{
    for (int i = 0; i < n; i++) out[i] = orc_tex2d1(t, xy[2 * i], xy[2 * i + 1]);
}
