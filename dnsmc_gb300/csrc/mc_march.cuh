// mc_march.cuh -- the device helpers of the marches (Philox, Sobol', the
// attenuation and trigonometric polynomials, table lookups, the control
// variate's straight flight, the ray's words, direction, slab and tally),
// the multigrid march (march_mg_kernel, instantiated in mc_kernels.cu) and
// the launch helpers; the fine-grid two-cell marches are in
// mc_march_pair.cuh.  The march translation units are compiled with
// -fmad=false: the arithmetic is written with explicit fmaf so the host
// replay (oracle/mc_oracle.cpp) reproduces every ray bit for bit; exp, log,
// sin and cos are the project's own polynomial kernels for the same reason.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "mc_internal.h"
#include "../../include/dnsmc.h"

namespace dnsmc {

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

// ---------------------------------------------------------------------------
// expm1 for x <= 0: Cody-Waite reduction x = n*ln2 + r, then expm1(r) =
// r (1 + r g(r)) with g(r) = (e^r - 1 - r)/r^2 replaced by its degree-4
// minimax polynomial on [-ln2/2, ln2/2] (Remez exchange computed for this
// project; |error| 6.2e-8 on g), then 2^n expm1(r) + (2^n - 1).  n is
// rounded by the shifter sh = fmaf(x, log2(e), 1.5 * 2^23): the sum lies in
// [2^23, 2^24), where the float spacing is 1, so sh - 1.5 * 2^23 is an
// integer within 1/2 (plus the fma's rounding) of x log2(e), and the low bits
// of sh hold n itself, so 2^n is one integer multiply-add on them.  Only +,
// *, fmaf and integer bit operations: bit-identical on any IEEE-754 machine.
// ---------------------------------------------------------------------------
constexpr float kExpShift = 12582912.0f;           // 1.5 * 2^23, bits 0x4B400000
__device__ __forceinline__ float mc_pow2_from_shift(float sh) {
    // bits(sh) = 0x4B400000 + n, so (n + 127) << 23 is bits(sh) << 23 plus a
    // constant, modulo 2^32
    return __uint_as_float((__float_as_uint(sh) << 23) + ((127u - 0x4B400000u) << 23));
}
__device__ __forceinline__ float mc_expm1(float x) {
    x = fmaxf(x, -87.0f);                          // n in [-126, 0]
    const float sh = fmaf(x, 1.44269504088896341f, kExpShift);
    const float n = sh - kExpShift;
    float r = fmaf(n, -0.693145751953125f, x);
    r = fmaf(n, -1.42860682030941723212e-6f, r);
    float q = 1.39411131385713816e-3f;
    q = fmaf(q, r, 8.36317520588636398e-3f);
    q = fmaf(q, r, 4.16663736104965210e-2f);
    q = fmaf(q, r, 1.66665762662887573e-1f);
    q = fmaf(q, r, 0.5f);
    float p = fmaf(q, r, 1.0f);
    p = p * r;                                     // expm1(r)
    const float two_n = mc_pow2_from_shift(sh);
    return fmaf(two_n, p, two_n - 1.0f);
}

// mc_expm1 of two arguments at once with paired FP32 instructions
// (f32x2 add / mul / fma, each half rounded to nearest like its scalar
// form): the same operations in the same order, so each half is
// bit-identical to mc_expm1 of it.  Used for the two cells of a lane.
__device__ __forceinline__ float2 mc_expm1_x2(float2 x) {
    x.x = fmaxf(x.x, -87.0f);
    x.y = fmaxf(x.y, -87.0f);
    const float2 sh = __ffma2_rn(x, make_float2(1.44269504088896341f, 1.44269504088896341f),
                                 make_float2(kExpShift, kExpShift));
    const float2 n = __fadd2_rn(sh, make_float2(-kExpShift, -kExpShift));
    float2 r = __ffma2_rn(n, make_float2(-0.693145751953125f, -0.693145751953125f), x);
    r = __ffma2_rn(n, make_float2(-1.42860682030941723212e-6f, -1.42860682030941723212e-6f), r);
    float2 q = __ffma2_rn(make_float2(1.39411131385713816e-3f, 1.39411131385713816e-3f), r,
                          make_float2(8.36317520588636398e-3f, 8.36317520588636398e-3f));
    q = __ffma2_rn(q, r, make_float2(4.16663736104965210e-2f, 4.16663736104965210e-2f));
    q = __ffma2_rn(q, r, make_float2(1.66665762662887573e-1f, 1.66665762662887573e-1f));
    q = __ffma2_rn(q, r, make_float2(0.5f, 0.5f));
    float2 p = __ffma2_rn(q, r, make_float2(1.0f, 1.0f));
    p = __fmul2_rn(p, r);
    const float2 two_n = make_float2(mc_pow2_from_shift(sh.x), mc_pow2_from_shift(sh.y));
    return __ffma2_rn(two_n, p, __fadd2_rn(two_n, make_float2(-1.0f, -1.0f)));
}

// sin and cos of x in [0, pi/4]: Taylor series to x^11 / x^12.
__device__ __forceinline__ void mc_sincos_oct(float x, float *s, float *c) {
    const float z = x * x;
    float ps = -2.50521083854417188e-8f;           // -1/11!
    ps = fmaf(ps, z, 2.75573192239858907e-6f);     //  1/9!
    ps = fmaf(ps, z, -1.98412698412698413e-4f);    // -1/7!
    ps = fmaf(ps, z, 8.33333333333333333e-3f);     //  1/5!
    ps = fmaf(ps, z, -1.66666666666666667e-1f);    // -1/3!
    *s = fmaf(ps * z, x, x);
    float pc = 2.08767569878680990e-9f;            //  1/12!
    pc = fmaf(pc, z, -2.75573192239858907e-7f);    // -1/10!
    pc = fmaf(pc, z, 2.48015873015873016e-5f);     //  1/8!
    pc = fmaf(pc, z, -1.38888888888888889e-3f);    // -1/6!
    pc = fmaf(pc, z, 4.16666666666666667e-2f);     //  1/4!
    pc = fmaf(pc, z, -0.5f);
    *c = fmaf(pc, z, 1.0f);
}

// cos and sin of 2*pi*m/2^24 for a 24-bit integer m: exact quadrant and
// octant reduction on the integer, polynomial on [0, pi/4].
__device__ __forceinline__ void mc_sincos_turn(uint32_t m, float *cs, float *sn) {
    const uint32_t q = m >> 22;
    const uint32_t r = m & 0x3FFFFFu;
    const bool hi = r > 0x200000u;
    const float th = (float)(hi ? (0x400000u - r) : r) * 3.74507028e-7f;  // pi*2^-23
    float s, c;
    mc_sincos_oct(th, &s, &c);
    const float cq = hi ? s : c, sq = hi ? c : s;
    float co, si;
    switch (q) {
        case 0: co = cq;  si = sq;  break;
        case 1: co = -sq; si = cq;  break;
        case 2: co = -cq; si = -sq; break;
        default: co = sq; si = -cq; break;
    }
    *cs = co; *sn = si;
}

// Sobol' direction numbers of the four sampled dimensions (host-computed).
static __constant__ uint32_t c_sobol[4][32];  // one copy per translation unit

__device__ __forceinline__ uint4 sobol4(uint32_t m) {
    uint32_t a = 0, b = 0, c = 0, d = 0;
    while (m) {  // one pass per set bit of m
        const int k = __ffs(m) - 1;
        a ^= c_sobol[0][k]; b ^= c_sobol[1][k]; c ^= c_sobol[2][k]; d ^= c_sobol[3][k];
        m &= m - 1u;
    }
    return make_uint4(a, b, c, d);
}

__device__ __forceinline__ float u24(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }

// Linear position in a uniform grid of n points, clamped as the reference's
// clamp-addressed linear-filter textures (code/memory_copy.cu:245-247).
__device__ __forceinline__ void grid_pos(float v, float v0, float inv, int n, int *i, float *f) {
    float p = (v - v0) * inv;
    p = fminf(fmaxf(p, 0.0f), (float)(n - 1));
    int ii = (int)p;
    ii = min(ii, n - 2);
    *i = ii;
    *f = p - (float)ii;
}

// Split a clamped table coordinate p in [0, n-1] into cell and fraction.
__device__ __forceinline__ void pos_split(float p, int n, int *i, float *f) {
    int ii = (int)p;
    ii = min(ii, n - 2);
    *i = ii;
    *f = p - (float)ii;
}

// Paired tables: the k part of a sample's slab holds, per table cell
// kidx = ti*(nX-1) + xi of an x-table, the 16-byte entry (k[t][x],
// k[t][x+1] - k[t][x], k[t+1][x], k[t+1][x+1] - k[t+1][x]) for t = ti <=
// nT - 2, or per ti the pair (k[t], k[t+1] - k[t]); its Ib part holds (Ib[t],
// Ib[t+1] - Ib[t]) of the sample's band.  A bilinear lookup is one 16-byte
// load and three fmaf (the differences are the same FP32 subtractions the
// interpolation would do).  The march reads them from the warp's copy of the
// slab in shared memory.
template <int MODE>
__device__ __forceinline__ float lookup_k(const float2 *ks, int kidx, float ft, float fx) {
    if (MODE == MODE_TX) {
        const float4 v = reinterpret_cast<const float4 *>(ks)[kidx];
        const float2 a = make_float2(v.x, v.y), b = make_float2(v.z, v.w);
        const float k0 = fmaf(fx, a.y, a.x);
        const float k1 = fmaf(fx, b.y, b.x);
        return fmaf(ft, k1 - k0, k0);
    } else {
        const float2 a = ks[kidx];
        return fmaf(ft, a.y, a.x);
    }
}

__device__ __forceinline__ float lookup_ib(const float2 *ibs, int ti, float ft) {
    const float2 a = ibs[ti];
    return fmaf(ft, a.y, a.x);
}

// Field element type of the march: T (grey), or the cell's table coordinates.
template <int MODE> struct FieldT { typedef float type; };
template <> struct FieldT<MODE_T> { typedef int2 type; };
template <> struct FieldT<MODE_TX> { typedef int4 type; };

// (k index, T cell, T fraction, x fraction) of a table-coordinate element
template <int MODE>
__device__ __forceinline__ void cell_coords(const typename FieldT<MODE>::type &v, int *kidx, int *ti, float *ft,
                                            float *fx) {
    if constexpr (MODE == MODE_TX) {
        *kidx = v.x; *ft = __int_as_float(v.y); *fx = __int_as_float(v.z); *ti = v.w;
    } else if constexpr (MODE == MODE_T) {
        *kidx = v.x; *ti = v.x; *ft = __int_as_float(v.y); *fx = 0.0f;
    }
}

template <int MODE>
__device__ __forceinline__ typename FieldT<MODE>::type load_field(const MarchParams &P, long long fbase, int cell) {
    if constexpr (MODE == MODE_TX) return __ldg(P.fieldPX + fbase + cell);
    else if constexpr (MODE == MODE_T) return __ldg(P.fieldP + fbase + cell);
    else return __ldg(P.fieldT + fbase + cell);
}

// ---------------------------------------------------------------------------
// -ln(u) for u in (0, 1): u = m 2^e with m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(s), s = (m - 1)/(m + 1), odd series to s^11 (|s| <= 0.1716,
// truncation below 1e-9); e ln 2 split Cody-Waite.  +, *, /, fmaf only.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float mc_neglog(float u) {
    uint32_t b = __float_as_uint(u);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = __uint_as_float((b & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float p = 9.09090909090909091e-2f;            // 1/11
    p = fmaf(p, z, 1.11111111111111111e-1f);       // 1/9
    p = fmaf(p, z, 1.42857142857142857e-1f);       // 1/7
    p = fmaf(p, z, 2.0e-1f);                       // 1/5
    p = fmaf(p, z, 3.33333333333333333e-1f);       // 1/3
    p = fmaf(p, z, 1.0f);
    const float lnm = 2.0f * s * p;
    const float fe = (float)e;
    const float ln = fmaf(fe, 0.693145751953125f, fmaf(fe, 1.42860682030941723212e-6f, lnm));
    return -ln;
}

// uniform in (0, 1) from the top 24 bits
__device__ __forceinline__ float u24o(uint32_t x) { return ((float)(x >> 8) + 0.5f) * 5.9604644775390625e-8f; }

// Direction scattered by the Henyey-Greenstein phase function (asymmetry g)
// from (sW, sA, sB): cos(theta) from uc, azimuth 2 pi m / 2^24.
__device__ __forceinline__ void hg_scatter(float g, uint32_t uc, uint32_t um, float *sW, float *sA, float *sB) {
    const float u = u24(uc);
    float ct;
    if (fabsf(g) < 1e-6f) {
        ct = 1.0f - 2.0f * u;
    } else {
        const float tmp = (1.0f - g * g) / (1.0f - g + 2.0f * g * u);
        ct = (1.0f + g * g - tmp * tmp) / (2.0f * g);
    }
    ct = fminf(fmaxf(ct, -1.0f), 1.0f);
    const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float cph, sph;
    mc_sincos_turn(um >> 8, &cph, &sph);
    const float w = *sW, a = *sA, b = *sB;
    float nw, na, nb;
    if (fabsf(w) > 0.99999f) {
        na = st * cph;
        nb = st * sph;
        nw = w > 0.0f ? ct : -ct;
    } else {
        const float tmp = sqrtf(1.0f - w * w);
        na = st * (a * w * cph - b * sph) / tmp + a * ct;
        nb = st * (b * w * cph + a * sph) / tmp + b * ct;
        nw = -st * cph * tmp + w * ct;
    }
    *sW = nw; *sA = na; *sB = nb;
}

// Surrogate of the control variate: the ray's straight flight through the
// layer-mean medium, read from its table row (the ray's field, spectral
// sample and layer; cv_table_kernel) by linear interpolation in
// u = sqrt(|sW|) between the nodes m / kSurBins.  Returns the collected
// intensity J and the own-layer absorptance A.  The reads are warp-uniform.
__device__ __forceinline__ void surrogate_lookup(const float4 *row, float sW, float *J, float *A) {
    const float x = sqrtf(fabsf(sW)) * (float)kSurBins;
    const int m = min((int)x, kSurBins - 1);
    const float r = x - (float)m;
    const float4 e = __ldg(row + (sW > 0.0f ? kSurBins : 0) + m);
    *J = fmaf(r, e.y, e.x);
    *A = fmaf(r, e.w, e.z);
}

// ---------------------------------------------------------------------------
// Pieces shared by the marches (the multigrid march below and the two-cell
// marches of mc_march_pair.cuh): the words of a packet-ray, its direction,
// the copy of its spectral sample's table slab, one ray's tally.
// ---------------------------------------------------------------------------

// The ray's four uniform words.  RQMC: point m of replicate b = r / M of a
// Sobol' net, XOR-shifted by the replicate's Philox word (kept in *shift and
// recomputed when the replicate changes, *bcur); iid: one Philox call.
__device__ __forceinline__ uint4 ray_words(const MarchParams &P, int r, int M, int p, uint32_t ctr2, int *bcur,
                                          uint4 *shift, int *m_out) {
    if (P.sampler) {
        const int b = r / M;
        const int m = r - b * M;
        if (b != *bcur) {
            *shift = philox4x32_10(make_uint4((uint32_t)b, (uint32_t)p, ctr2, 0x50B01u), P.key0, P.key1);
            *bcur = b;
        }
        const uint4 sh = *shift;
        const uint4 sb = sobol4((uint32_t)m);
        *m_out = m;
        return make_uint4(sb.x ^ sh.x, sb.y ^ sh.y, sb.z ^ sh.z, sb.w ^ sh.w);
    }
    *m_out = 0;
    return philox4x32_10(make_uint4((uint32_t)r, (uint32_t)p, ctr2, 0u), P.key0, P.key1);
}

// Isotropic direction (the reference's emiss_ang, code/mc_gpu.cu:813-820):
// cos(theta) = 1 - 2u from the top 24 bits of x.y, phi = 2 pi u' from x.x.
__device__ __forceinline__ void ray_direction(uint4 x, float *sW, float *sA, float *sB) {
    const float mu = fmaf((float)(x.y >> 8), -1.1920928955078125e-7f, 1.0f);
    const float st = sqrtf(fmaxf(0.0f, fmaf(-mu, mu, 1.0f)));
    float cph, sph;
    mc_sincos_turn(x.x >> 8, &cph, &sph);
    *sW = mu;
    *sA = st * cph;
    *sB = st * sph;
}

// ---------------------------------------------------------------------------
// The ray's table slab arrives by one bulk copy of the TMA engine
// (cp.async.bulk, global -> this CTA's shared memory) that signals the warp's
// transaction barrier (mbarrier) in shared memory; the warp waits on the
// barrier's phase parity.  Each warp owns one barrier and one slab buffer.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Lane 0 initialises the warp's barrier (one arrival per phase: the issuing
// lane's arrive.expect_tx) before the warp's first copy.
__device__ __forceinline__ void slab_bar_init(uint64_t *bar, int lane) {
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
}

// Bounded wait (at most `polls` polls) for the barrier phase of the given
// parity to complete.
__device__ __forceinline__ bool slab_bar_wait(const uint64_t *bar, uint32_t parity, int polls) {
    const uint32_t b = smem_addr(bar);
    for (int it = 0; it < polls; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(b), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// The sample's slab (k, then Ib of its band; slab_len * 8 bytes, a multiple
// of 16 at a 16-byte aligned address on both sides) into this warp's shared
// copy.  The previous ray's lookups are done first (the warp converges, and
// the async proxy is ordered after the generic one).  *phase is the warp's
// barrier parity, flipped per completed copy.  The first wait polls
// P.slab_polls0 times (kSlabWaitPolls; fewer only in tests of this path).
// A wait that runs out sets DNSMC_STATUS_COPY_TIMEOUT (the host reports the
// solve as failed) and waits once more; if the copy has still not arrived,
// returns false with the phase unchanged: the warp then takes no further
// copies or items and calls slab_drain before it exits.  The outcome is
// the same in every lane of the warp.
__device__ __forceinline__ bool load_slab(const MarchParams &P, int sid, float2 *slk, int lane, uint64_t *bar,
                                          uint32_t *phase, unsigned int *flags) {
    __syncwarp();
    if (lane == 0) {
        const uint32_t bytes = (uint32_t)P.slab_len * 8u;
        const float2 *src = P.slab + (long long)sid * P.slab_len;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(slk)),
                     "l"(src), "r"(bytes), "r"(smem_addr(bar))
                     : "memory");
    }
    if (!__all_sync(0xffffffffu, slab_bar_wait(bar, *phase, P.slab_polls0))) {
        *flags |= DNSMC_STATUS_COPY_TIMEOUT;
        if (!__all_sync(0xffffffffu, slab_bar_wait(bar, *phase, kSlabWaitPolls))) return false;
    }
    *phase ^= 1u;
    return true;
}

// Before a warp whose copy did not arrive exits: one more bounded wait for
// that copy, so that it does not land in shared memory the next block on
// this SM may own.
__device__ __forceinline__ void slab_drain(const uint64_t *bar, uint32_t phase) {
    slab_bar_wait(bar, phase, kSlabWaitPolls);
}

// Float pairs (hi, lo): about 48 bits at FP32 rates (error-free sums; the
// translation units of the marches are compiled without FMA contraction, so
// the error terms stay exact).  This GPU's FP64 rate is a small fraction of
// its FP32 rate, and a warp's FP64 instructions at the end of every ray
// held the march up.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    const float s = a.x + b.x;
    const float bb = s - a.x;
    float e = (a.x - (s - bb)) + (b.x - bb);
    e = e + (a.y + b.y);
    const float hi = s + e;
    return make_float2(hi, e - (hi - s));
}
__device__ __forceinline__ float2 ff_addf(float2 a, float b) {
    const float s = a.x + b;
    const float bb = s - a.x;
    float e = (a.x - (s - bb)) + (b - bb);
    e = e + a.y;
    const float hi = s + e;
    return make_float2(hi, e - (hi - s));
}
__device__ __forceinline__ double ff_value(float2 a) { return (double)a.x + (double)a.y; }

// One ray of a cell into its sums, as float pairs: the sum, and the sum of
// squares (iid) or of the squared replicate means (RQMC: *rep holds the
// running replicate sum, m the ray's index in its replicate of M rays; the
// mean is the pair divided by M, its remainder exact by fma).
__device__ __forceinline__ void tally_ray(const MarchParams &P, float X, int m, int M, float2 *sum, float2 *sq,
                                          float2 *rep) {
    *sum = ff_addf(*sum, X);
    if (P.sampler) {
        const float2 Sb = ff_addf(*rep, X);
        if (m == M - 1) {  // end of a replicate: accumulate its mean squared
            const float Mf = (float)M;
            const float q = Sb.x / Mf;
            const float ql = (fmaf(-q, Mf, Sb.x) + Sb.y) / Mf;
            const float p = q * q;
            *sq = ff_add(*sq, make_float2(p, fmaf(q, q, -p) + 2.0f * (q * ql)));
            *rep = make_float2(0.0f, 0.0f);
        } else {
            *rep = Sb;
        }
    } else {
        const float p = X * X;
        *sq = ff_add(*sq, make_float2(p, fmaf(X, X, -p)));
    }
}

// ---------------------------------------------------------------------------
// The multigrid march (grid_num > 1; the reference's grid switch,
// code/mc_gpu.cu:193-207), one cell per lane, 32-cell packets: the absorbing
// gas with black walls, grey or T tables, no control variate.  Persistent:
// every warp pulls work items (field, band group, packet) from an atomic
// counter.  The fine phase is the warp-uniform walk of the two-cell march
// (mc_march_pair.cuh) for mg_steps steps; then every lane continues from its
// own point on the coarser grids with the reference's position-update march.
// ---------------------------------------------------------------------------
// Resident blocks of 256 threads per SM the register allocation must allow
// (2: up to 128 registers; 3: 85; 4: 64), chosen at build time.
#ifndef DNSMC_MINB
#define DNSMC_MINB 4
#endif
template <int MODE, bool TRACE>
__global__ void __launch_bounds__(256, DNSMC_MINB) march_mg_kernel(const MarchParams P) {
    typedef typename FieldT<MODE>::type VT;
    const unsigned FULL = 0xffffffffu;
    const float INF = __int_as_float(0x7f800000);
    const int lane = threadIdx.x & 31;
    const int la = lane % P.tile_a, lb = lane / P.tile_a;
    const int njR = P.ea1 - P.ea0, nkR = P.eb1 - P.eb0;
    const int plane = P.na * P.nb;
    unsigned long long my_rays = 0, my_steps = 0;
    unsigned int flags = 0;
    const int tid = threadIdx.x;
    // dynamic shared memory (march_smem, one cell per lane): this warp's copy
    // of the current ray's table slab (tabulated models), the item's sums as
    // float pairs [3][threads] and the replicate's shift [threads]
    extern __shared__ float4 s_dyn[];
    const int nthr = blockDim.x;
    float2 *const slk = reinterpret_cast<float2 *>(s_dyn) + (threadIdx.x >> 5) * P.slab_len;
    const float2 *const sli = slk + P.slab_klen;
    double *const s_acc = reinterpret_cast<double *>(reinterpret_cast<float2 *>(s_dyn) + ((nthr + 31) >> 5) * P.slab_len);
    uint4 *const s_shift = reinterpret_cast<uint4 *>(s_acc + 3 * nthr);
    // each warp's transaction barrier of its slab copies, and its parity
    __shared__ uint64_t s_bar[8];
    uint64_t *const sbar = &s_bar[threadIdx.x >> 5];
    uint32_t sphase = 0;
    slab_bar_init(sbar, lane);
    bool dead = false;  // a slab copy did not arrive: this warp stops marching

    for (;;) {
        long long item;
        if (TRACE) {
            if (threadIdx.x >= 32) return;
            item = ((long long)P.trace_f * P.n_groups + P.trace_g) * P.n_packets + P.trace_p;
        } else {
            unsigned int it = 0;
            if (lane == 0) it = atomicAdd(P.queue, 1u);
            it = __shfl_sync(FULL, it, 0);
            if ((long long)it >= P.n_items) break;
            item = P.item_order ? (long long)__ldg(P.item_order + it) : (long long)it;
        }
        const int p = (int)(item % P.n_packets);
        const long long fg = item / P.n_packets;
        const int G = (int)(fg % P.n_groups);
        const int f = (int)(fg / P.n_groups);
        const int pa = p % P.npa;
        const int rest = p / P.npa;
        const int pb = rest % P.npb;
        const int pw = rest / P.npb;
        const int w0 = P.ew0 + pw;
        const int a0 = P.ea0 + pa * P.tile_a + la;
        const int b0 = P.eb0 + pb * P.tile_b + lb;
        const bool active = (a0 < P.ea1) && (b0 < P.eb1);
        const int acl = active ? a0 : P.ea0, bcl = active ? b0 : P.eb0;
        const int N = P.rays_per_packet ? P.rays_per_packet[G * P.rays_gstride + p] : P.rays;
        const long long fbase = (long long)f * P.field_stride;
        const int rowW0 = w0 * plane;
        // own-cell quantities
        const VT vown = load_field<MODE>(P, fbase, rowW0 + bcl * P.na + acl);
        float Ti4 = 0.f, tpos0 = 0.f;
        int ti_i = 0, ki_i = 0;
        float ft_i = 0.f, fx_i = 0.f;
        if constexpr (MODE == MODE_GREY) {
            const float Ti = vown;
            if (!(Ti > 0.0f) && active) flags |= DNSMC_STATUS_BAD_FIELD;
            const float t2 = Ti * Ti;
            Ti4 = t2 * t2;
        } else {
            cell_coords<MODE>(vown, &ki_i, &ti_i, &ft_i, &fx_i);
            tpos0 = (float)ti_i + ft_i;  // the clamped table coordinate, exactly
        }
        const float oW = (__ldg(P.fw + w0) + __ldg(P.fw + w0 + 1)) * 0.5f;
        // alias table of this packet: band group G of the temperature bin
        // nearest to lane 0's temperature (one bin when sampling at Tmax)
        int gs = 0, K = 1;
        if (MODE != MODE_GREY) {
            int boff = 0;
            if (P.n_tbins > 1) {
                const float tp0 = __shfl_sync(FULL, tpos0, 0);
                int bin = __float2int_rn(tp0);
                bin = min(max(bin, 0), P.n_tbins - 1);
                boff = bin * P.n_groups;
            }
            gs = P.group_start[boff + G];
            K = P.group_start[boff + G + 1] - gs;
        }
        const uint32_t ctr2 = (uint32_t)G | ((uint32_t)(f + P.field_base) << 16);
        const long long tc = ((long long)(w0 - P.ew0) * nkR + (bcl - P.eb0)) * njR + (acl - P.ea0);
        const long long cell_out = fg * P.region_cells + tc;  // tally index of this lane's cell
        const int M = P.sampler ? max(1, N / max(1, P.nbatch)) : 1;
        s_acc[tid] = 0.0; s_acc[nthr + tid] = 0.0; s_acc[2 * nthr + tid] = 0.0;
        unsigned long long isteps = 0;
        unsigned int lsteps = 0;  // this lane's active steps in the item
        int bcur = -1;
        const int rbeg = TRACE ? P.trace_r : 0;
        const int rend = TRACE ? P.trace_r + 1 : ((K > 0) ? N : 0);
        for (int r = rbeg; r < rend; ++r) {
            int m;
            const uint4 x = ray_words(P, r, M, p, ctr2, &bcur, &s_shift[tid], &m);
            if (TRACE && lane == 0) {
                P.trace_rng[0] = x.x; P.trace_rng[1] = x.y; P.trace_rng[2] = x.z; P.trace_rng[3] = x.w;
            }
            float sW, sA, sB;
            ray_direction(x, &sW, &sA, &sB);

            // spectral sample and ray weight (the ray contributes wk D, D the
            // net exchange in intensity units)
            float wk, Ii;
            int nbnd = 0;
            if (MODE == MODE_GREY) {
                Ii = Ti4;
                wk = P.Wgrey;
            } else {
                const int j = (int)__umulhi(x.z, (uint32_t)K);
                SpecEntry e = P.entries[gs + j];
                if (!(u24(x.w) < e.prob)) e = P.entries[gs + (int)(e.alias_nb & 0xFFFFu)];
                nbnd = (int)(e.alias_nb >> 16);
                if (!load_slab(P, e.koff, slk, lane, sbar, &sphase, &flags)) { dead = true; break; }
                const float ki = lookup_k<MODE>(slk, ki_i, ft_i, fx_i);
                Ii = lookup_ib(sli, ti_i, ft_i);
                wk = e.W * ki;
            }

            // fine phase: the warp-uniform DDA from the cell centres
            const float invW = 1.0f / fabsf(sW), invA = 1.0f / fabsf(sA), invB = 1.0f / fabsf(sB);
            const int dW = sW > 0.f ? 1 : -1, dA = sA > 0.f ? 1 : -1, dB = sB > 0.f ? 1 : -1;
            int cw = w0, ca = acl, cb = bcl;
            float tW = (dW > 0 ? (__ldg(P.fw + cw + 1) - oW) : (oW - __ldg(P.fw + cw))) * invW;
            const float dtA = P.da * invA, dtB = P.db * invB;
            float tA = 0.5f * dtA, tB = 0.5f * dtB;
            int nA = 0, nB = 0;
            float t = 0.0f;
            int rowW = rowW0, rowB = cb * P.na;
            float tau = active ? 1.0f : 0.0f;
            float D = 0.0f;
            int steps = 0;
            VT vcur = vown;
            for (;;) {
                int axis;
                float tn;
                if (tW <= tA && tW <= tB) { axis = 0; tn = tW; }
                else if (tA <= tB)         { axis = 1; tn = tA; }
                else                       { axis = 2; tn = tB; }
                const float ds = tn - t;
                // next cell of the walk, and its field value fetched now
                int ncw = cw, nca = ca, ncb = cb, nrowW = rowW, nrowB = rowB;
                bool wall = false;
                if (axis == 0) {
                    ncw = cw + dW;
                    wall = ncw < 0 || ncw >= P.nw;
                    nrowW = ncw * plane;
                } else if (axis == 1) {
                    nca = ca + dA;
                    if (nca == P.na) nca = 0; else if (nca < 0) nca = P.na - 1;
                } else {
                    ncb = cb + dB;
                    if (ncb == P.nb) ncb = 0; else if (ncb < 0) ncb = P.nb - 1;
                    nrowB = ncb * P.na;
                }
                VT vnext = vcur;
                if (!wall && tau > 0.0f) vnext = load_field<MODE>(P, fbase, nrowW + nrowB + nca);
                if (tau > 0.0f) {
                    ++lsteps;
                    float kj, gj;
                    if constexpr (MODE == MODE_GREY) {
                        const float t2 = vcur * vcur;
                        gj = Ti4 - t2 * t2;
                        kj = P.kappa;
                    } else {
                        int kx, tj;
                        float ftj, fxj;
                        cell_coords<MODE>(vcur, &kx, &tj, &ftj, &fxj);
                        kj = lookup_k<MODE>(slk, kx, ftj, fxj);
                        const float Ibj = lookup_ib(sli, tj, ftj);
                        gj = Ii - Ibj;
                    }
                    const float alpha = -mc_expm1(-(kj * ds));
                    const float ta = tau * alpha;
                    D = fmaf(ta, gj, D);
                    tau = tau - ta;
                    if (tau < P.toll) { D = fmaf(tau, gj, D); tau = 0.0f; }
                }
                if (TRACE && lane == 0 && steps < P.trace_max) {
                    int *rec = P.trace_rec + 6 * steps;
                    rec[0] = cw; rec[1] = dA * nA; rec[2] = dB * nB; rec[3] = axis;
                    rec[4] = __float_as_int(ds); rec[5] = __float_as_int(tau);
                }
                t = tn;
                ++steps;
                if (axis == 0) {
                    if (wall) {
                        const int side = ncw < 0 ? 0 : 1;
                        const float Iw = (MODE == MODE_GREY) ? P.Tw4[side] : __ldg(P.ibw + side * P.nbands + nbnd);
                        if (tau > 0.0f) {
                            D = fmaf(tau, Ii - Iw, D);
                            tau = 0.0f;
                        }
                        break;
                    }
                    cw = ncw;
                    rowW = nrowW;
                    tW = (dW > 0 ? (__ldg(P.fw + cw + 1) - oW) : (oW - __ldg(P.fw + cw))) * invW;
                } else if (axis == 1) {
                    ++nA;
                    tA = ((float)nA + 0.5f) * dtA;
                    ca = nca;
                } else {
                    ++nB;
                    tB = ((float)nB + 0.5f) * dtB;
                    cb = ncb;
                    rowB = nrowB;
                }
                vcur = vnext;
                if (!__any_sync(FULL, tau > 0.0f)) break;
                if (steps >= P.mg_steps) break;
            }
            {
                // Coarse grids (the reference's grid switch, code/mc_gpu.cu:193-207):
                // every lane continues from its own point with the reference's
                // position-update march; lanes no longer share their cell
                // faces, but they step in lockstep and leave a level together.
                if (__any_sync(FULL, tau > 0.0f)) {
                    const float ua = t / dtA - (float)nA, ub = t / dtB - (float)nB;
                    const float fa = fminf(fmaxf(dA > 0 ? 0.5f + ua : 0.5f - ua, 0.0f), 1.0f);
                    const float fb = fminf(fmaxf(dB > 0 ? 0.5f + ub : 0.5f - ub, 0.0f), 1.0f);
                    float xp = fmaf(sW, t, oW);
                    float yp = ((float)ca + fa) * P.da;
                    float zp = ((float)cb + fb) * P.db;
                    int ic = cw, jc = ca, kc = cb;
                    const float isx = 1.0f / sW, isy = 1.0f / sA, isz = 1.0f / sB;
                    int counter = 0, cap = 0;
                    for (int l = 1; l < P.mg_levels; ++l) {
                        ic >>= 1; jc >>= 1; kc >>= 1;
                        const int nwL = P.nw >> l, naL = P.na >> l, nbL = P.nb >> l;
                        const float *fwL = P.mgfw + P.mg_fwoff[l];
                        const float daL = P.mg_da[l], dbL = P.mg_db[l];
                        const float *TL = P.mgT + P.mg_off[l] + (long long)f * nwL * naL * nbL;
                        cap = (l == P.mg_levels - 1) ? P.max_steps : P.mg_steps;
                        counter = 0;
                        while (__any_sync(FULL, tau > 0.0f && counter < cap)) {
                            float dsr = 0.0f;  // this lane's segment (0 when it idles)
                            if (tau > 0.0f && counter < cap) {
                                const float fx = __ldg(fwL + (dW > 0 ? ic + 1 : ic));
                                const float fy = (float)(dA > 0 ? jc + 1 : jc) * daL;
                                const float fz = (float)(dB > 0 ? kc + 1 : kc) * dbL;
                                const float dsx = sW != 0.0f ? (fx - xp) * isx : INF;
                                const float dsy = sA != 0.0f ? (fy - yp) * isy : INF;
                                const float dsz = sB != 0.0f ? (fz - zp) * isz : INF;
                                const float Tc = __ldg(TL + ((long long)ic * nbL + kc) * naL + jc);
                                float kj, gj;
                                if constexpr (MODE == MODE_GREY) {
                                    const float t2 = Tc * Tc;
                                    gj = Ti4 - t2 * t2;
                                    kj = P.kappa;
                                } else {
                                    float pt = (Tc - P.T0) * P.invdT;
                                    pt = fminf(fmaxf(pt, 0.0f), (float)(P.nT - 1));
                                    int tj;
                                    float ftj;
                                    pos_split(pt, P.nT, &tj, &ftj);
                                    kj = lookup_k<MODE_T>(slk, tj, ftj, 0.0f);
                                    gj = Ii - lookup_ib(sli, tj, ftj);
                                }
                                float dmin = dsx;
                                if (dmin > dsy) dmin = dsy;
                                if (dmin > dsz) dmin = dsz;
                                const float ds = fmaxf(dmin, 0.0f);
                                dsr = ds;
                                xp = (dmin == dsx) ? fx : fmaf(ds, sW, xp);
                                yp = (dmin == dsy) ? fy : fmaf(ds, sA, yp);
                                zp = (dmin == dsz) ? fz : fmaf(ds, sB, zp);
                                const float alpha = -mc_expm1(-(kj * ds));
                                const float ta = tau * alpha;
                                D = fmaf(ta, gj, D);
                                tau = tau - ta;
                                if (tau < P.toll) { D = fmaf(tau, gj, D); tau = 0.0f; }
                                int axis;
                                if (dsx < dsy) axis = (dsx < dsz) ? 0 : 2;
                                else axis = (dsy < dsz) ? 1 : 2;
                                if (axis == 0) {
                                    ic += dW;
                                    if (ic < 0 || ic >= nwL) {
                                        const int side = ic < 0 ? 0 : 1;
                                        const float Iw = (MODE == MODE_GREY) ? P.Tw4[side]
                                                                             : __ldg(P.ibw + side * P.nbands + nbnd);
                                        if (tau > 0.0f) D = fmaf(tau, Ii - Iw, D);
                                        tau = 0.0f;
                                        ic = ic < 0 ? 0 : nwL - 1;
                                    }
                                } else if (axis == 1) {
                                    jc += dA;
                                    if (jc >= naL) { jc = 0; yp = 0.0f; } else if (jc < 0) { jc = naL - 1; yp = P.Ly; }
                                } else {
                                    kc += dB;
                                    if (kc >= nbL) { kc = 0; zp = 0.0f; } else if (kc < 0) { kc = nbL - 1; zp = P.Lz; }
                                }
                                ++lsteps;
                            }
                            if (TRACE && lane == 0 && steps < P.trace_max) {  // every iteration
                                int *rec = P.trace_rec + 6 * steps;
                                rec[0] = ic; rec[1] = jc; rec[2] = kc; rec[3] = 16 + l;
                                rec[4] = __float_as_int(dsr); rec[5] = __float_as_int(tau);
                            }
                            ++counter;
                            ++steps;
                        }
                    }
                    if (tau > 0.0f) flags |= DNSMC_STATUS_STEP_CAP;
                }
            }
            if (TRACE && lane == 0) *P.trace_n = steps;
            isteps += (unsigned long long)steps;
            const float X = wk * D;
            if (active) {
                ++my_rays;
                if (!isfinite(X)) flags |= DNSMC_STATUS_NONFINITE;
                tally_ray(P, X, m, M, reinterpret_cast<float2 *>(&s_acc[tid]), reinterpret_cast<float2 *>(&s_acc[nthr + tid]),
                          reinterpret_cast<float2 *>(&s_acc[2 * nthr + tid]));
            }
        }
        if (dead) break;  // the item's sums are incomplete; the solve fails
        my_steps += lsteps;
        if (TRACE) return;
        if (P.item_steps && lane == 0) P.item_steps[item] = isteps;
        if (active)
            P.tally[cell_out] = make_double2(ff_value(*reinterpret_cast<const float2 *>(&s_acc[tid])),
                                             ff_value(*reinterpret_cast<const float2 *>(&s_acc[nthr + tid])));
    }
    if (dead) slab_drain(sbar, sphase);
    // per-warp counters and status
    for (int o = 16; o > 0; o >>= 1) {
        my_rays += __shfl_xor_sync(FULL, my_rays, o);
        my_steps += __shfl_xor_sync(FULL, my_steps, o);
        flags |= __shfl_xor_sync(FULL, flags, o);
    }
    if (lane == 0) {
        if (my_rays) atomicAdd(P.counters + 0, my_rays);
        if (my_steps) atomicAdd(P.counters + 1, my_steps);
        if (flags) atomicOr(P.status, flags);
    }
}

// Dynamic shared memory of a march kernel: a kernel whose static plus
// dynamic shared memory exceeds the default 48 KB per block needs its limit
// raised once (queried first, so a launch inside a graph capture only reads).
inline int march_prepare_smem(void (*k)(const MarchParams), size_t smem) {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k);
    if (e != cudaSuccess) return (int)e;
    if (fa.sharedSizeBytes + smem > 48u * 1024u && (size_t)fa.maxDynamicSharedSizeBytes < smem)
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return (int)e;
}

// One launch of a march kernel with `smem` bytes of dynamic shared memory,
// and its resident blocks per SM.
inline int march_launch_one(void (*k)(const MarchParams), int blocks, int threads, size_t smem, cudaStream_t st,
                            const MarchParams &p) {
    if (const int e = march_prepare_smem(k, smem)) return e;
    dnsmc::note_launch();
    k<<<blocks, threads, smem, st>>>(p);
    return (int)cudaGetLastError();
}

inline int march_occupancy_one(void (*k)(const MarchParams), int threads, size_t smem) {
    if (march_prepare_smem(k, smem)) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, threads, smem) != cudaSuccess) return 0;
    return nb;
}

}  // namespace dnsmc
