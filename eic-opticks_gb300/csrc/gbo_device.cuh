// gbo_device.cuh : device-side vector helpers, the counter-based Philox stream and photon bit packing.
//
// Arithmetic follows the reference device code operation by operation (binary32, nvcc default contraction)
// so that flag histories agree with the reference GPU path:
//   float3 helpers       sysrap/scuda.h:519-606 (normalize multiplies by 1/sqrtf, float3/float by reciprocal)
//   Philox4x32-10        Random123 (Salmon et al., SC'11); stream layout of curand_init(seed, subsequence,
//                        offset) + skipahead(skipahead_event_offset*event) (qudarap/qrng.h:131-137)
//   sphoton packing      sysrap/sphoton.h:171-231, set_prd :482-488
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/gbo_types.h"

#define GBO_DEV __device__ __forceinline__
// a branch taken by few photons of any workload (reemission, Rayleigh scattering, diffuse reflection): the compiler
// lays its code out of the straight path of a step
#define GBO_UNLIKELY(c) __builtin_expect(!!(c), 0)

namespace gbo {

// ---- float3 --------------------------------------------------------------------------------------------------
GBO_DEV float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
GBO_DEV float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
GBO_DEV float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
GBO_DEV float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
GBO_DEV float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
GBO_DEV float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
GBO_DEV float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
GBO_DEV float3 divs(float3 a, float s) { float inv = 1.0f / s; return a * inv; }
GBO_DEV float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GBO_DEV float3 cross(float3 a, float3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
GBO_DEV float length(float3 a) { return sqrtf(dot(a, a)); }
GBO_DEV float3 normalize(float3 a) { float inv = 1.0f / sqrtf(dot(a, a)); return a * inv; }
GBO_DEV float3 fminf3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
GBO_DEV float3 fmaxf3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }

constexpr float PI_F = 3.14159265358979323846f;

// ---- Philox4x32-10, stateless counter form ------------------------------------------------------------------
// A photon's stream position p (draws consumed so far, including the offset and event skipahead) maps to the
// 128-bit counter (p >> 2, subsequence) and output lane p & 3 : the layout curand's Philox state walks.
// Blocks are computed lazily: skip() only moves the position, so a block whose four outputs are all
// alignment "burn" draws of the reference is never computed.
// CALL selects how a block is computed: false inlines the ten rounds at every draw site, true calls one
// out-of-line block function.  The photon program draws at dozens of sites; inlined rounds at each of them make the
// CSG-tree kernels large enough to miss in the instruction cache (20,000-sensor event 156M -> 172M photons/s with the
// call), while the single-leaf kernel of the crystal event runs faster inlined (845M vs 784M photons/s).  Both give
// the same numbers.
template <bool CALL>
struct RngT {
    uint64_t pos;         // draws consumed (position in the subsequence)
    uint64_t cached;      // block index held in out[], ~0 when none
    uint32_t sub_lo, sub_hi;
    uint32_t key0, key1;
    uint32_t out[4];
};

GBO_DEV void philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t* o)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c0;
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    o[0] = c0; o[1] = c1; o[2] = c2; o[3] = c3;
}

template <bool CALL>
GBO_DEV void rng_init(RngT<CALL>& r, uint64_t seed, uint64_t subsequence, uint64_t position)
{
    r.key0 = (uint32_t)seed;
    r.key1 = (uint32_t)(seed >> 32);
    r.sub_lo = (uint32_t)subsequence;
    r.sub_hi = (uint32_t)(subsequence >> 32);
    r.pos = position;
    r.cached = ~0ull;
}

template <bool CALL>
GBO_DEV void skip(RngT<CALL>& r, unsigned n) { r.pos += n; }

// One Philox block out of line (RngT<true>): arguments and result travel in registers (no address is taken), and the
// call runs once per four draws.
static __device__ __noinline__ uint4 philox_block(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
    uint32_t o[4];
    philox10(c0, c1, c2, c3, k0, k1, o);
    return make_uint4(o[0], o[1], o[2], o[3]);
}

template <bool CALL>
GBO_DEV float uniform(RngT<CALL>& r)
{
    const uint64_t b = r.pos >> 2;
    if (b != r.cached) {
        if constexpr (CALL) {
            const uint4 o = philox_block((uint32_t)b, (uint32_t)(b >> 32), r.sub_lo, r.sub_hi, r.key0, r.key1);
            r.out[0] = o.x; r.out[1] = o.y; r.out[2] = o.z; r.out[3] = o.w;
        } else {
            philox10((uint32_t)b, (uint32_t)(b >> 32), r.sub_lo, r.sub_hi, r.key0, r.key1, r.out);
        }
        r.cached = b;
    }
    uint32_t x;
    switch ((unsigned)r.pos & 3u) {  // explicit select keeps out[] in registers
        case 0: x = r.out[0]; break;
        case 1: x = r.out[1]; break;
        case 2: x = r.out[2]; break;
        default: x = r.out[3]; break;
    }
    r.pos += 1;
    return (float)x * 2.3283064365386963e-10f + (2.3283064365386963e-10f / 2.0f);
}

// ---- photon record in registers ------------------------------------------------------------------------------
struct Photon {
    float3 pos; float time;
    float3 mom; uint32_t hitcount_iindex;
    float3 pol; float wavelength;
    uint32_t orient_boundary_flag, identity, index, flagmask;
};

GBO_DEV unsigned flag_of(const Photon& p) { return p.orient_boundary_flag & 0xffffu; }
GBO_DEV unsigned boundary_of(const Photon& p) { return (p.orient_boundary_flag & 0x7fff0000u) >> 16; }
GBO_DEV void set_flag(Photon& p, unsigned f)
{
    p.orient_boundary_flag = (p.orient_boundary_flag & 0xffff0000u) | (f & 0xffffu);
    p.flagmask |= f;
}
GBO_DEV void zero_flags(Photon& p)
{
    p.orient_boundary_flag = 0u; p.identity = 0u; p.index = 0u; p.flagmask = 0u; p.hitcount_iindex = 0u;
}
GBO_DEV void set_prd(Photon& p, unsigned boundary, unsigned identity, float orient, unsigned iindex)
{
    p.orient_boundary_flag = (p.orient_boundary_flag & 0x8000ffffu) | ((boundary & 0x7fffu) << 16);
    p.identity = (p.identity & 0xff000000u) | (identity & 0x00ffffffu);
    p.orient_boundary_flag = (p.orient_boundary_flag & 0x7fffffffu) | ((orient < 0.f ? 0x1u : 0x0u) << 31);
    p.hitcount_iindex = 0x00010000u | (0x0000ffffu & iindex);
}
GBO_DEV void set_index(Photon& p, uint64_t full)
{
    p.index = (uint32_t)(full & 0xffffffffu);
    p.identity = ((uint32_t)((full >> 32) & 0xffu) << 24) | (p.identity & 0xffffffu);
}

GBO_DEV void load_photon(Photon& p, const gbo_sphoton* s)
{
    const float4* q = reinterpret_cast<const float4*>(s);
    float4 a = q[0], b = q[1], c = q[2], d = q[3];
    p.pos = f3(a.x, a.y, a.z); p.time = a.w;
    p.mom = f3(b.x, b.y, b.z); p.hitcount_iindex = __float_as_uint(b.w);
    p.pol = f3(c.x, c.y, c.z); p.wavelength = c.w;
    p.orient_boundary_flag = __float_as_uint(d.x); p.identity = __float_as_uint(d.y);
    p.index = __float_as_uint(d.z); p.flagmask = __float_as_uint(d.w);
}

// the same through L2 only (ld.global.cg): streamed photons read once do not displace the L1-resident geometry and
// boundary texture lines
GBO_DEV void load_photon_streamed(Photon& p, const gbo_sphoton* s)
{
    const float4* q = reinterpret_cast<const float4*>(s);
    const float4 a = __ldcg(q), b = __ldcg(q + 1), c = __ldcg(q + 2), d = __ldcg(q + 3);
    p.pos = f3(a.x, a.y, a.z); p.time = a.w;
    p.mom = f3(b.x, b.y, b.z); p.hitcount_iindex = __float_as_uint(b.w);
    p.pol = f3(c.x, c.y, c.z); p.wavelength = c.w;
    p.orient_boundary_flag = __float_as_uint(d.x); p.identity = __float_as_uint(d.y);
    p.index = __float_as_uint(d.z); p.flagmask = __float_as_uint(d.w);
}

GBO_DEV void store_photon(gbo_sphoton* s, const Photon& p)
{
    float4* q = reinterpret_cast<float4*>(s);
    q[0] = make_float4(p.pos.x, p.pos.y, p.pos.z, p.time);
    q[1] = make_float4(p.mom.x, p.mom.y, p.mom.z, __uint_as_float(p.hitcount_iindex));
    q[2] = make_float4(p.pol.x, p.pol.y, p.pol.z, p.wavelength);
    q[3] = make_float4(__uint_as_float(p.orient_boundary_flag), __uint_as_float(p.identity),
                       __uint_as_float(p.index), __uint_as_float(p.flagmask));
}

// photon history nibbles : sysrap/sseq.h:174-184.  The record is kept in its output slot in device memory (a
// debug output): the simulation loop then holds no registers for it when recording is off.
GBO_DEV void seq_add(gbo_seq* q, unsigned slot, unsigned flag, unsigned boundary)
{
    const unsigned iseq = slot / 16u;
    const unsigned shift = 4u * (slot - iseq * 16u);
    if (iseq < 2u) {
        q->seqhis[iseq] |= ((unsigned long long)(__ffs((int)flag) & 0xf)) << shift;
        q->seqbnd[iseq] |= ((unsigned long long)(boundary & 0xfu)) << shift;
    }
}
GBO_DEV void seq_start(gbo_seq* q, unsigned flag, unsigned boundary)
{
    q->seqhis[0] = q->seqhis[1] = q->seqbnd[0] = q->seqbnd[1] = 0ull;
    seq_add(q, 0u, flag, boundary);
}

}  // namespace gbo
