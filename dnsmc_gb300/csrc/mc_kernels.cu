// mc_kernels.cu -- sm_103a device code of the reverse (emission-based, OERM)
// Monte Carlo radiative-source solver.
//
// Replaces kernel_fluid / march_ray / find_band / emiss_ang / kernel_results
// of the reference (code/mc_gpu.cu:44-438, :813-896, :959-970) with one
// persistent work-queue kernel built around "packets":
//
//   * a packet is 32 cells that share the wall-normal index i and tile the
//     periodic (j, k) plane (tile_a x tile_b, j fastest in memory);
//   * one warp owns a packet; lane l owns cell l and keeps that cell's FP64
//     tallies in registers, so no reduction is needed;
//   * every ray of the packet shares one Philox draw: the isotropic direction
//     (reference emiss_ang, code/mc_gpu.cu:813-820) and the spectral sample
//     (band, g) drawn from an alias table (reference find_band, :830-896).
//     The reference already shares its Sobol direction sequence across all
//     cells (code/mc_gpu.cu:80-81).  Because the origins differ by whole
//     periodic cells, the voxel walk (which face is crossed next, and the
//     segment length) is identical in all 32 lanes: the DDA is warp-uniform,
//     lanes only offset their (j, k) indices.  Field gathers of the 32 lanes
//     are contiguous (256 B per step for float2 fields) and the spectral
//     table slice is the same for the whole warp.
//   * per segment each lane does the OERM update of march_ray
//     (code/mc_gpu.cu:264-276): alpha = 1 - exp(-k ds),
//     D += tau*alpha*(Ib_i - Ib_j)/Ib_i, tau *= 1 - alpha, the remainder is
//     dumped when tau < toll, black walls add tau*(Ib_i - Ib_w)/Ib_i
//     (code/mc_gpu.cu:297,314).  The ray contribution is X = W*k_i*Ib_i*D.
//
// Rays are drawn either iid (one Philox4x32-10 call per packet-ray) or as
// randomised quasi-Monte Carlo: the N rays of a (packet, band group) are
// nbatch replicates of the first N/nbatch points of a 4-dimensional Sobol' net
// (phi, cos theta, spectral index, alias threshold), each replicate XOR-shifted
// by a Philox word; the spectral sample comes from the alias table of the
// packet's own temperature bin when local sampling is on.
//
// Arithmetic is FP32 with explicit fmaf and the file is compiled with
// -fmad=false, so the host replay reproduces every ray bit for bit; exp and
// sin/cos are the project's own polynomial kernels (mc_expm1 / mc_sincos) for
// the same reason.  Tallies (sum X, sum X^2) are FP64.
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
// expm1 for x <= 0: Cody-Waite reduction x = n*ln2 + r, |r| <= ln2/2, Taylor
// series of expm1(r) to r^8/8!, then 2^n*expm1(r) + (2^n - 1).  Only +, *,
// fmaf and rintf: bit-identical on any IEEE-754 machine.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float mc_expm1(float x) {
    x = fmaxf(x, -87.0f);
    const float n = rintf(x * 1.44269504088896341f);
    float r = fmaf(-n, 0.693145751953125f, x);
    r = fmaf(-n, 1.42860682030941723212e-6f, r);
    float p = 2.48015873015873016e-5f;             // 1/8!
    p = fmaf(p, r, 1.98412698412698413e-4f);       // 1/7!
    p = fmaf(p, r, 1.38888888888888889e-3f);       // 1/6!
    p = fmaf(p, r, 8.33333333333333333e-3f);       // 1/5!
    p = fmaf(p, r, 4.16666666666666667e-2f);       // 1/4!
    p = fmaf(p, r, 1.66666666666666667e-1f);       // 1/3!
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = p * r;                                     // expm1(r)
    const int ni = (int)n;                         // in [-126, 0]
    const float two_n = __int_as_float((ni + 127) << 23);
    return fmaf(two_n, p, two_n - 1.0f);
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
__constant__ uint32_t c_sobol[4][32];

__device__ __forceinline__ uint4 sobol4(uint32_t m) {
    uint32_t a = 0, b = 0, c = 0, d = 0;
    for (int k = 0; m; ++k, m >>= 1)
        if (m & 1u) { a ^= c_sobol[0][k]; b ^= c_sobol[1][k]; c ^= c_sobol[2][k]; d ^= c_sobol[3][k]; }
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

// Paired tables: kpair holds (k[t][x], k[t][x+1]) (x-tables) or (k[t], k[t+1])
// and ibpair (Ib[t], Ib[t+1]), so a bilinear lookup is two 8-byte loads.
template <int MODE>
__device__ __forceinline__ float lookup_k(const MarchParams &P, int sid, int ti, float ft, int xi, float fx) {
    if (MODE == MODE_TX) {
        const int row = P.nX - 1;
        const float2 *r = P.kpair + (sid * P.nT + ti) * row + xi;
        const float2 a = __ldg(r), b = __ldg(r + row);
        const float k0 = fmaf(fx, a.y - a.x, a.x);
        const float k1 = fmaf(fx, b.y - b.x, b.x);
        return fmaf(ft, k1 - k0, k0);
    } else {
        const float2 a = __ldg(P.kpair + sid * (P.nT - 1) + ti);
        return fmaf(ft, a.y - a.x, a.x);
    }
}

__device__ __forceinline__ float lookup_ib(const MarchParams &P, int nb, int ti, float ft) {
    const float2 a = __ldg(P.ibpair + nb * (P.nT - 1) + ti);
    return fmaf(ft, a.y - a.x, a.x);
}

// Field element type of the march: T (grey), table T coordinate, or (T, x) coordinates.
template <int MODE> struct FieldT { typedef float type; };
template <> struct FieldT<MODE_TX> { typedef float2 type; };

template <int MODE>
__device__ __forceinline__ typename FieldT<MODE>::type load_field(const MarchParams &P, long long fbase, int cell) {
    if constexpr (MODE == MODE_TX) return __ldg(P.fieldPX + fbase + cell);
    else if constexpr (MODE == MODE_T) return __ldg(P.fieldP + fbase + cell);
    else return __ldg(P.fieldT + fbase + cell);
}

// ---------------------------------------------------------------------------
// The march kernel.  Persistent: every warp pulls work items (field, band
// group, packet) from an atomic counter until the queue is empty.  The next
// cell's field value is loaded one step ahead of its use.
// ---------------------------------------------------------------------------
// Resident blocks of 256 threads per SM the register allocation must allow
// (2: up to 128 registers; 3: 85; 4: 64), chosen at build time.
#ifndef DNSMC_MINB
#define DNSMC_MINB 4
#endif

template <int MODE, bool TRACE, bool CV, bool MOM = false>
__global__ void __launch_bounds__(256, DNSMC_MINB) march_kernel(const MarchParams P) {
    typedef typename FieldT<MODE>::type VT;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int la = lane % P.tile_a, lb = lane / P.tile_a;
    const int njR = P.ea1 - P.ea0, nkR = P.eb1 - P.eb0;
    const int plane = P.na * P.nb;
    unsigned long long my_rays = 0, my_steps = 0;
    unsigned int flags = 0;

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
            item = it;
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
        float Ti4 = 0.f, invTi4 = 0.f, tpos0 = 0.f;
        int ti_i = 0, xi_i = 0;
        float ft_i = 0.f, fx_i = 0.f;
        if constexpr (MODE == MODE_GREY) {
            const float Ti = vown;
            if (!(Ti > 0.0f) && active) flags |= DNSMC_STATUS_BAD_FIELD;
            const float t2 = Ti * Ti;
            Ti4 = t2 * t2;
            invTi4 = Ti4 > 0.f ? 1.0f / Ti4 : 0.f;
        } else if constexpr (MODE == MODE_TX) {
            tpos0 = vown.x;
            pos_split(vown.x, P.nT, &ti_i, &ft_i);
            pos_split(vown.y, P.nX, &xi_i, &fx_i);
        } else {
            tpos0 = vown;
            pos_split(vown, P.nT, &ti_i, &ft_i);
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
        float2 beta = make_float2(1.0f, -1.0f);
        if (CV && P.beta) beta = P.beta[fg * P.region_cells + tc];
        double mo[9];
        if (MOM)
#pragma unroll
            for (int q = 0; q < 9; ++q) mo[q] = 0.0;
        const int M = P.sampler ? max(1, N / max(1, P.nbatch)) : 1;

        double S = 0.0, S2 = 0.0, Sb = 0.0;
        unsigned long long isteps = 0;
        uint4 shift = make_uint4(0u, 0u, 0u, 0u);
        int bcur = -1;
        const int rbeg = TRACE ? P.trace_r : 0;
        const int rend = TRACE ? P.trace_r + 1 : ((K > 0) ? N : 0);
        for (int r = rbeg; r < rend; ++r) {
            uint4 x;
            int m = 0;
            if (P.sampler) {
                const int b = r / M;
                m = r - b * M;
                if (b != bcur) {
                    shift = philox4x32_10(make_uint4((uint32_t)b, (uint32_t)p, ctr2, 0x50B01u), P.key0, P.key1);
                    bcur = b;
                }
                const uint4 sb = sobol4((uint32_t)m);
                x = make_uint4(sb.x ^ shift.x, sb.y ^ shift.y, sb.z ^ shift.z, sb.w ^ shift.w);
            } else {
                x = philox4x32_10(make_uint4((uint32_t)r, (uint32_t)p, ctr2, 0u), P.key0, P.key1);
            }
            if (TRACE && lane == 0) {
                P.trace_rng[0] = x.x; P.trace_rng[1] = x.y; P.trace_rng[2] = x.z; P.trace_rng[3] = x.w;
            }
            // isotropic direction: cos(theta) = 1 - 2u, phi = 2*pi*u'
            const float mu = fmaf((float)(x.y >> 8), -1.1920928955078125e-7f, 1.0f);
            const float st = sqrtf(fmaxf(0.0f, fmaf(-mu, mu, 1.0f)));
            float cph, sph;
            mc_sincos_turn(x.x >> 8, &cph, &sph);
            const float sW = mu, sA = st * cph, sB = st * sph;

            // spectral sample and ray weight
            float w, wk, Ii, invI;
            int nbnd = 0, sid = 0;
            if (MODE == MODE_GREY) {
                Ii = Ti4;
                invI = invTi4;
                wk = P.Wgrey;
                w = P.Wgrey * Ti4;
            } else {
                const int j = (int)__umulhi(x.z, (uint32_t)K);
                SpecEntry e = P.entries[gs + j];
                if (!(u24(x.w) < e.prob)) e = P.entries[gs + (int)(e.alias_nb & 0xFFFFu)];
                nbnd = (int)(e.alias_nb >> 16);
                sid = e.koff;
                const float ki = lookup_k<MODE>(P, sid, ti_i, ft_i, xi_i, fx_i);
                Ii = lookup_ib(P, nbnd, ti_i, ft_i);
                invI = Ii > 0.f ? 1.0f / Ii : 0.f;
                wk = e.W * ki;
                w = wk * Ii;
            }
            // surrogate walk (warp-uniform): the same ray through the
            // layer-mean medium.  Its k and Ib are constant inside a wall-
            // normal layer, so it is advanced once per layer: tauE and tE are
            // its transmissivity and ray parameter at the layer entry, dcumE
            // the optical depth from the origin; it stops (dumping the rest
            // into the current layer) once the optical depth exceeds ln(1/toll).
            const float2 *surp = nullptr;
            float Jbar = 0.0f, tex0 = -1.0f, tauE = 0.0f, tE = 0.0f, dcumE = 0.0f, kS = 0.0f, IS = 0.0f, I0 = 0.0f;
            bool salive = false;
            if (CV) {
                surp = P.sur + ((long long)f * P.n_samples + sid) * P.nw;
                const float2 kv = __ldg(surp + w0);
                kS = kv.x; IS = kv.y; I0 = kv.y;
                tauE = 1.0f;
                salive = true;
            }

            // warp-uniform DDA set-up (origin at the cell centre)
            const float invW = 1.0f / fabsf(sW), invA = 1.0f / fabsf(sA), invB = 1.0f / fabsf(sB);
            const int dW = sW > 0.f ? 1 : -1, dA = sA > 0.f ? 1 : -1, dB = sB > 0.f ? 1 : -1;
            float tW = (dW > 0 ? (__ldg(P.fw + w0 + 1) - oW) : (oW - __ldg(P.fw + w0))) * invW;
            const float dtA = P.da * invA, dtB = P.db * invB;
            float tA = 0.5f * dtA, tB = 0.5f * dtB;
            int nA = 0, nB = 0;
            float t = 0.0f;
            int cw = w0, ca = acl, cb = bcl;
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
                    ++my_steps;
                    float kj, gj;
                    if constexpr (MODE == MODE_GREY) {
                        const float t2 = vcur * vcur;
                        gj = (Ti4 - t2 * t2) * invI;
                        kj = P.kappa;
                    } else {
                        int tj, xj = 0;
                        float ftj, fxj = 0.f;
                        if constexpr (MODE == MODE_TX) {
                            pos_split(vcur.x, P.nT, &tj, &ftj);
                            pos_split(vcur.y, P.nX, &xj, &fxj);
                        } else {
                            pos_split(vcur, P.nT, &tj, &ftj);
                        }
                        kj = lookup_k<MODE>(P, sid, tj, ftj, xj, fxj);
                        const float Ibj = lookup_ib(P, nbnd, tj, ftj);
                        gj = (Ii - Ibj) * invI;
                    }
                    const float alpha = -mc_expm1(-(kj * ds));
                    const float ta = tau * alpha;
                    D = fmaf(ta, gj, D);
                    tau = tau - ta;
                    if (tau < P.toll) { D = fmaf(tau, gj, D); tau = 0.0f; }
                }
                if (CV && salive) {
                    const float opt = kS * (tn - tE);
                    if (dcumE + opt > P.dtoll) {          // truncated inside this layer
                        Jbar = fmaf(tauE, IS, Jbar);
                        salive = false;
                    } else if (axis == 0) {               // leaves the layer at tn
                        const float as = -mc_expm1(-opt);
                        const float tas = tauE * as;
                        Jbar = fmaf(tas, IS, Jbar);
                        tauE = tauE - tas;
                        dcumE = dcumE + opt;
                        tE = tn;
                        if (tex0 < 0.0f) tex0 = tauE;     // transmissivity leaving the own layer
                        if (!wall) {
                            const float2 kv = __ldg(surp + ncw);
                            kS = kv.x; IS = kv.y;
                        }
                    }
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
                            D = fmaf(tau, (Ii - Iw) * invI, D);
                            tau = 0.0f;
                        }
                        if (CV && salive) {
                            Jbar = fmaf(tauE, Iw, Jbar);
                            salive = false;
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
                if (!__any_sync(FULL, tau > 0.0f || (CV && salive))) break;
                if (steps >= P.max_steps) {
                    if (tau > 0.0f || (CV && salive)) flags |= DNSMC_STATUS_STEP_CAP;
                    break;
                }
            }
            if (TRACE && lane == 0) *P.trace_n = steps;
            isteps += (unsigned long long)steps;
            float X = w * D;
            if (CV) {
                // Y_a: the ray through the layer-mean medium; Y_b: its own-layer part
                const float te = tex0 < 0.0f ? 0.0f : tex0;
                const float Ya = wk * (Ii - Jbar);
                const float Yb = wk * ((1.0f - te) * (Ii - I0));
                if (MOM && active) {
                    const double xd = X, ya = Ya, yb = Yb;
                    mo[0] += xd; mo[1] += ya; mo[2] += yb;
                    mo[3] = fma(xd, xd, mo[3]); mo[4] = fma(ya, ya, mo[4]); mo[5] = fma(yb, yb, mo[5]);
                    mo[6] = fma(xd, ya, mo[6]); mo[7] = fma(xd, yb, mo[7]); mo[8] = fma(ya, yb, mo[8]);
                }
                X = X - beta.x * Ya;  // tallied: X - beta_a Y_a - beta_b Y_b; the
                X = X - beta.y * Yb;  // means beta . E[Y] are added back at finalize
            }
            if (active) {
                ++my_rays;
                if (!isfinite(X)) flags |= DNSMC_STATUS_NONFINITE;
                const double Xd = (double)X;
                S += Xd;
                if (P.sampler) {
                    Sb += Xd;
                    if (m == M - 1) {  // end of a replicate: accumulate its mean squared
                        const double mb = Sb / M;
                        S2 = fma(mb, mb, S2);
                        Sb = 0.0;
                    }
                } else {
                    S2 = fma(Xd, Xd, S2);
                }
            }
        }
        if (TRACE) return;
        if (P.item_steps && lane == 0) P.item_steps[item] = isteps;
        if (active) P.tally[fg * P.region_cells + tc] = make_double2(S, S2);
        if (MOM && active) {
            double *out = P.moments + (fg * P.region_cells + tc) * 9;
#pragma unroll
            for (int q = 0; q < 9; ++q) out[q] = mo[q];
        }
    }
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

// Table coordinates of the field for the march: p = clamp((T - T0)/dT, 0,
// nT-1) (and the same for x_H2O), computed once per solve with the same FP32
// operations the march used to apply per step.
__global__ void field_pos_kernel(const float *fT, const float2 *fTX, float *outP, float2 *outPX, long long n,
                                 float T0, float invdT, int nT, float X0, float invdX, int nX) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        if (fTX) {
            const float2 v = fTX[i];
            float pt = (v.x - T0) * invdT;
            pt = fminf(fmaxf(pt, 0.0f), (float)(nT - 1));
            float px = (v.y - X0) * invdX;
            px = fminf(fmaxf(px, 0.0f), (float)(nX - 1));
            outPX[i] = make_float2(pt, px);
        } else {
            float pt = (fT[i] - T0) * invdT;
            pt = fminf(fmaxf(pt, 0.0f), (float)(nT - 1));
            outP[i] = pt;
        }
    }
}

// ---------------------------------------------------------------------------
// Finalize: per cell of the region, Q = sum over groups of the group means,
// var(Q) = sum of the variances of the group means (groups are independent
// strata).  Replaces kernel_results + the host scatter (code/mc_gpu.cu:959-970,
// :762-776); the output is dense, i fastest.
// ---------------------------------------------------------------------------
__global__ void finalize_kernel(const FinalizeParams F) {
    const long long n = (long long)F.nfields * F.region_cells;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(idx / F.region_cells);
        const long long c = idx - (long long)f * F.region_cells;
        const int iR = (int)(c % F.niR);
        const long long jk = c / F.niR;
        const int jR = (int)(jk % F.njR);
        const int kR = (int)(jk / F.njR);
        const long long tc = ((long long)iR * F.nkR + kR) * F.njR + jR;
        const int p = (iR * F.npb + kR / F.tile_b) * F.npa + jR / F.tile_a;
        double Q = 0.0, V = 0.0;
        for (int g = 0; g < F.n_groups; ++g) {
            const int N = F.rays_per_packet ? F.rays_per_packet[g * F.rays_gstride + p] : F.rays;
            double m = 0.0, v = 0.0;
            if (!F.group_empty[g] && N > 0) {
                const long long ti = ((long long)f * F.n_groups + g) * F.region_cells + tc;
                const double2 t = F.tally[ti];
                m = t.x / N;
                if (F.batched) {
                    const int B = F.nbatch;
                    if (B > 1) v = fmax(0.0, t.y / B - m * m) / (B - 1);
                } else if (N > 1) {
                    v = fmax(0.0, t.y / N - m * m) / (N - 1);
                }
            }
            if (F.muY && !F.group_empty[g]) {
                const long long ti = ((long long)f * F.n_groups + g) * F.region_cells + tc;
                const float2 b = F.beta ? F.beta[ti] : make_float2(1.0f, -1.0f);
                const double2 mu = F.muY[ti];
                // Q_g = beta_a E[Y_a] + beta_b E[Y_b] + mean(X - beta_a Y_a - beta_b Y_b)
                m += (double)b.x * mu.x;
                m += (double)b.y * mu.y;
            }
            Q += m;
            V += v;
            if (F.Qg) {
                const long long o = ((long long)f * F.n_groups + g) * F.region_cells + c;
                F.Qg[o] = m;
                F.varg[o] = v;
            }
        }
        F.Q[idx] = Q;
        F.var[idx] = V;
    }
}

// Transpose a host-order field (i fastest, optional ghost layer) into the
// device order [i][k][j].  One thread per destination cell.
__global__ void pack_T_kernel(const float *src, float *dst, int nw, int na, int nb,
                              long long si, long long sj, long long sk, long long base) {
    const long long n = (long long)nw * na * nb;
    for (long long d = blockIdx.x * (long long)blockDim.x + threadIdx.x; d < n;
         d += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(d % na);
        const long long r = d / na;
        const int b = (int)(r % nb);
        const int w = (int)(r / nb);
        dst[d] = src[base + w * si + a * sj + b * sk];
    }
}

__global__ void pack_TX_kernel(const float *srcT, const float *srcX, float2 *dst, int nw, int na,
                               int nb, long long si, long long sj, long long sk, long long base) {
    const long long n = (long long)nw * na * nb;
    for (long long d = blockIdx.x * (long long)blockDim.x + threadIdx.x; d < n;
         d += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(d % na);
        const long long r = d / na;
        const int b = (int)(r % nb);
        const int w = (int)(r / nb);
        const long long s = base + w * si + a * sj + b * sk;
        dst[d] = make_float2(srcT[s], srcX ? srcX[s] : 0.0f);
    }
}

// Deterministic two-pass reduction: max T, min T, sum x (fixed block count,
// fixed order), used when fields arrive as device pointers.
constexpr int kStatBlocks = 256, kStatThreads = 256;
__global__ void field_stats_pass1(const float *fT, const float2 *fTX, long long n, double *part) {
    __shared__ double smax[kStatThreads], smin[kStatThreads], ssum[kStatThreads];
    double mx = -1e300, mn = 1e300, sm = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float T, x = 0.f;
        if (fTX) { const float2 v = fTX[i]; T = v.x; x = v.y; } else { T = fT[i]; }
        mx = fmax(mx, (double)T); mn = fmin(mn, (double)T); sm += x;
    }
    smax[threadIdx.x] = mx; smin[threadIdx.x] = mn; ssum[threadIdx.x] = sm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = smax[0]; part[3 * blockIdx.x + 1] = smin[0]; part[3 * blockIdx.x + 2] = ssum[0];
    }
}
__global__ void field_stats_pass2(const double *part, int nparts, float *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double mx = -1e300, mn = 1e300, sm = 0.0;
    for (int i = 0; i < nparts; ++i) {
        mx = fmax(mx, part[3 * i]); mn = fmin(mn, part[3 * i + 1]); sm += part[3 * i + 2];
    }
    out[0] = (float)mx; out[1] = (float)mn; out[2] = (float)sm;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 4096) b = 4096;
    if (b < 1) b = 1;
    return (int)b;
}

int launch_march(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace) {
    cudaStream_t st = (cudaStream_t)stream;
    if (trace) { blocks = 1; threads = 32; }
    switch (mode) {
        case MODE_GREY:
            if (trace) march_kernel<MODE_GREY, true, false><<<blocks, threads, 0, st>>>(p);
            else march_kernel<MODE_GREY, false, false><<<blocks, threads, 0, st>>>(p);
            break;
        case MODE_T:
            if (trace) march_kernel<MODE_T, true, false><<<blocks, threads, 0, st>>>(p);
            else march_kernel<MODE_T, false, false><<<blocks, threads, 0, st>>>(p);
            break;
        case MODE_TX:
            if (trace) march_kernel<MODE_TX, true, false><<<blocks, threads, 0, st>>>(p);
            else march_kernel<MODE_TX, false, false><<<blocks, threads, 0, st>>>(p);
            break;
        default:
            return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

int launch_march_cv(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace,
                    bool moments) {
    cudaStream_t st = (cudaStream_t)stream;
    if (trace) { blocks = 1; threads = 32; }
    if (moments && !trace) {
        switch (mode) {
            case MODE_GREY: march_kernel<MODE_GREY, false, true, true><<<blocks, threads, 0, st>>>(p); break;
            case MODE_T: march_kernel<MODE_T, false, true, true><<<blocks, threads, 0, st>>>(p); break;
            case MODE_TX: march_kernel<MODE_TX, false, true, true><<<blocks, threads, 0, st>>>(p); break;
            default: return (int)cudaErrorInvalidValue;
        }
        return (int)cudaGetLastError();
    }
    switch (mode) {
        case MODE_GREY:
            if (trace) march_kernel<MODE_GREY, true, true><<<blocks, threads, 0, st>>>(p);
            else march_kernel<MODE_GREY, false, true><<<blocks, threads, 0, st>>>(p);
            break;
        case MODE_T:
            if (trace) march_kernel<MODE_T, true, true><<<blocks, threads, 0, st>>>(p);
            else march_kernel<MODE_T, false, true><<<blocks, threads, 0, st>>>(p);
            break;
        case MODE_TX:
            if (trace) march_kernel<MODE_TX, true, true><<<blocks, threads, 0, st>>>(p);
            else march_kernel<MODE_TX, false, true><<<blocks, threads, 0, st>>>(p);
            break;
        default:
            return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

int march_cv_occupancy(int mode, int threads, bool moments) {
    int nb = 0;
    cudaError_t e = cudaErrorInvalidValue;
    if (moments) {
        if (mode == MODE_GREY) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_GREY, false, true, true>, threads, 0);
        if (mode == MODE_T) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_T, false, true, true>, threads, 0);
        if (mode == MODE_TX) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_TX, false, true, true>, threads, 0);
        if (e != cudaSuccess) return 1;
        return nb > 0 ? nb : 1;
    }
    if (mode == MODE_GREY) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_GREY, false, true>, threads, 0);
    if (mode == MODE_T) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_T, false, true>, threads, 0);
    if (mode == MODE_TX) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_TX, false, true>, threads, 0);
    if (e != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

// ---------------------------------------------------------------------------
// Control variate preparation.  Y is the ray's contribution in the medium
// whose temperature and x_H2O are the mean of each wall-normal plane; its
// expectation per cell is a 1-D layered-slab integral:
//   E[Y] = sum_s C_s k_i(s) (Ib_i(s) - Jhat_s(layer)),
//   Jhat_s(l) = 1/2 int_{-1}^{1} J_s(mu; l) dmu,
// J_s the intensity absorbed along a ray leaving the centre of layer l with
// wall-normal cosine mu through the layer-mean medium (same toll cut-off,
// same wall emission).  The march tallies X - beta*Y and finalize adds
// beta*E[Y] back, so the estimate is unbiased for any beta.
// ---------------------------------------------------------------------------
__constant__ double c_quad_mu[128];
__constant__ double c_quad_w[128];
__constant__ int c_nquad;

int upload_quadrature(const double *mu, const double *w, int n) {
    cudaError_t e = cudaMemcpyToSymbol(c_quad_mu, mu, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_quad_w, w, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_nquad, &n, sizeof(int));
    return (int)e;
}

__device__ __forceinline__ float cv_k(const CvParams &c, int sid, float T, float x) {
    int ti, xi = 0;
    float ft, fx = 0.f;
    grid_pos(T, c.T0, c.invdT, c.nT, &ti, &ft);
    if (c.mode == MODE_TX) {
        grid_pos(x, c.X0, c.invdX, c.nX, &xi, &fx);
        const float *s = c.ktab + (long long)sid * c.nT * c.nX + ti * c.nX + xi;
        const float k00 = __ldg(s), k01 = __ldg(s + 1);
        const float k10 = __ldg(s + c.nX), k11 = __ldg(s + c.nX + 1);
        const float k0 = fmaf(fx, k01 - k00, k00);
        const float k1 = fmaf(fx, k11 - k10, k10);
        return fmaf(ft, k1 - k0, k0);
    }
    const float *s = c.ktab + (long long)sid * c.nT + ti;
    const float k0 = __ldg(s), k1 = __ldg(s + 1);
    return fmaf(ft, k1 - k0, k0);
}

__device__ __forceinline__ float cv_ib(const CvParams &c, int band, float T) {
    int ti;
    float ft;
    grid_pos(T, c.T0, c.invdT, c.nT, &ti, &ft);
    const float *s = c.ibtab + band * c.nT + ti;
    const float i0 = __ldg(s), i1 = __ldg(s + 1);
    return fmaf(ft, i1 - i0, i0);
}

// (T_bar, x_bar) of every wall-normal plane, fixed-order reduction.
__global__ void cv_layer_kernel(const CvParams c) {
    const int w = blockIdx.x, f = blockIdx.y;
    const long long plane = (long long)c.na * c.nb;
    const long long base = ((long long)f * c.nw + w) * plane;
    __shared__ double sT[256], sX[256];
    double aT = 0.0, aX = 0.0;
    for (long long i = threadIdx.x; i < plane; i += blockDim.x) {
        if (c.mode == MODE_TX) { const float2 v = c.fieldTX[base + i]; aT += v.x; aX += v.y; }
        else aT += c.fieldT[base + i];
    }
    sT[threadIdx.x] = aT;
    sX[threadIdx.x] = aX;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) { sT[threadIdx.x] += sT[threadIdx.x + o]; sX[threadIdx.x] += sX[threadIdx.x + o]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) c.layer[(long long)f * c.nw + w] = make_float2((float)(sT[0] / plane), (float)(sX[0] / plane));
}

// Layer-mean absorption coefficient and band intensity per (field, sample, layer).
__global__ void cv_sur_kernel(const CvParams c) {
    const long long n = (long long)c.nfields * c.n_samples * c.nw;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int w = (int)(idx % c.nw);
        const long long fs = idx / c.nw;
        const int sid = (int)(fs % c.n_samples);
        const int f = (int)(fs / c.n_samples);
        const float2 L = c.layer[(long long)f * c.nw + w];
        float kb, Ib;
        if (c.mode == MODE_GREY) {
            const float t2 = L.x * L.x;
            kb = c.kappa;
            Ib = t2 * t2;
        } else {
            kb = cv_k(c, sid, L.x, L.y);
            Ib = cv_ib(c, sid / c.nq, L.x);
        }
        c.sur[idx] = make_float2(kb, Ib);
    }
}

// Direction-averaged surrogate intensity Jhat per (field, sample, layer):
// composite Gauss-Legendre in mu on each hemisphere, 1-D march through the
// layers with the same toll cut-off and wall emission as the 3-D walk.
__global__ void cv_jhat_kernel(const CvParams c) {
    const long long n = (long long)c.nfields * c.n_samples * c.nw;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int w = (int)(idx % c.nw);
        const long long fs = idx / c.nw;
        const int sid = (int)(fs % c.n_samples);
        const float2 *sp = c.sur + fs * c.nw;
        const int band = c.mode == MODE_GREY ? 0 : sid / c.nq;
        const float oW = (__ldg(c.fw + w) + __ldg(c.fw + w + 1)) * 0.5f;
        double acc = 0.0, accA = 0.0;
        for (int h = 0; h < 2; ++h) {
            const int dir = h ? 1 : -1;
            const float Iw = c.mode == MODE_GREY ? c.Tw4[h] : __ldg(c.ibw + h * c.nbands + band);
            for (int q = 0; q < c_nquad; ++q) {
                const float inv_mu = (float)(1.0 / c_quad_mu[q]);
                float tau = 1.0f, J = 0.0f, t0 = 0.0f, dcum = 0.0f;
                int l = w;
                float seg = dir > 0 ? (__ldg(c.fw + w + 1) - oW) : (oW - __ldg(c.fw + w));
                for (;;) {
                    const float2 kv = sp[l];
                    const float opt = kv.x * seg * inv_mu;
                    if (dcum + opt > c.dtoll) { J = fmaf(tau, kv.y, J); break; }  // truncated in layer l
                    const float a = -expm1f(-opt);
                    const float ta = tau * a;
                    J = fmaf(ta, kv.y, J);
                    tau = tau - ta;
                    dcum = dcum + opt;
                    if (l == w) t0 = tau;  // transmissivity leaving the own layer
                    l += dir;
                    if (l < 0 || l >= c.nw) { J = fmaf(tau, Iw, J); break; }
                    seg = __ldg(c.fw + l + 1) - __ldg(c.fw + l);
                }
                acc += c_quad_w[q] * (double)J;
                accA += c_quad_w[q] * (1.0 - (double)t0);
            }
        }
        const double J = 0.5 * acc;
        const float Jhi = (float)J;
        c.Jhat[idx] = make_double2(J, 0.5 * accA);
        c.Jf[idx] = make_float4(Jhi, (float)(J - (double)Jhi), (float)(0.5 * accA), sp[w].y);
    }
}

// Compensated FP32 accumulation (Kahan): sum - comp carries the exact sum to
// about 2^-44 relative; the file is compiled without FMA contraction, so the
// compensation is not folded away.
struct KahanF {
    float s = 0.0f, comp = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - comp;
        const float t = s + y;
        comp = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)comp; }
};

// E[Y] per (field, group, cell of the region), tally layout [f][g][i][k][j]:
//   E[Y_a] = sum_s C_s k_s(T_i, x_i) (Ib_s(T_i) - Jhat_s(layer)),
//   E[Y_b] = sum_s C_s k_s(T_i, x_i) (Ib_s(T_i) - Ibar_s(layer)) Ahat_s(layer),
// over the group's spectral samples, in FP32 with compensated sums (the
// device's FP64 rate is a small fraction of its FP32 rate); Jhat enters as a
// double-float pair so Ib - Jhat keeps its digits where they cancel.
__global__ void cv_mean_kernel(const CvParams c) {
    const int njR = c.ea1 - c.ea0, nkR = c.eb1 - c.eb0;
    const long long n = (long long)c.nfields * c.region_cells;
    const long long plane = (long long)c.na * c.nb;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(idx / c.region_cells);
        const long long tc = idx - (long long)f * c.region_cells;
        const int jR = (int)(tc % njR);
        const long long r = tc / njR;
        const int kR = (int)(r % nkR);
        const int iR = (int)(r / nkR);
        const int w = c.ew0 + iR;
        const long long cell = (long long)f * c.nw * plane + (long long)w * plane + (long long)(c.eb0 + kR) * c.na + (c.ea0 + jR);
        float T, x = 0.f;
        if (c.mode == MODE_TX) { const float2 v = c.fieldTX[cell]; T = v.x; x = v.y; }
        else T = c.fieldT[cell];
        const long long sbase = (long long)f * c.n_samples * c.nw + w;
        if (c.mode == MODE_GREY) {
            const float t2 = T * T;
            const double2 jh = c.Jhat[sbase];
            const double acc = c.Wgrey * ((double)(t2 * t2) - jh.x);
            const double accB = c.Wgrey * ((double)(t2 * t2) - (double)c.sur[sbase].y) * jh.y;
            c.muY[(long long)f * c.n_groups * c.region_cells + tc] = make_double2(acc, accB);
            continue;
        }
        int ti, xi = 0;
        float ft, fx = 0.f;
        grid_pos(T, c.T0, c.invdT, c.nT, &ti, &ft);
        if (c.mode == MODE_TX) grid_pos(x, c.X0, c.invdX, c.nX, &xi, &fx);
        for (int g = 0; g < c.n_groups; ++g) {
            KahanF sa, sb;
            for (int q = c.grp_start[g]; q < c.grp_start[g + 1]; ++q) {
                const int sid = c.samp_id[q];
                float k;
                if (c.mode == MODE_TX) {
                    const float *s = c.ktab + (long long)sid * c.nT * c.nX + ti * c.nX + xi;
                    const float k00 = __ldg(s), k01 = __ldg(s + 1);
                    const float k10 = __ldg(s + c.nX), k11 = __ldg(s + c.nX + 1);
                    const float k0 = fmaf(fx, k01 - k00, k00);
                    const float k1 = fmaf(fx, k11 - k10, k10);
                    k = fmaf(ft, k1 - k0, k0);
                } else {
                    const float *s = c.ktab + (long long)sid * c.nT + ti;
                    const float k0 = __ldg(s), k1 = __ldg(s + 1);
                    k = fmaf(ft, k1 - k0, k0);
                }
                const float *ib = c.ibtab + (sid / c.nq) * c.nT + ti;
                const float i0 = __ldg(ib), i1 = __ldg(ib + 1);
                const float Ib = fmaf(ft, i1 - i0, i0);
                const float4 J = __ldg(c.Jf + sbase + (long long)sid * c.nw);
                const float ck = __ldg(c.samp_Cf + q) * k;
                sa.add(ck * ((Ib - J.x) - J.y));
                sb.add(ck * (Ib - J.w) * J.z);
            }
            c.muY[((long long)f * c.n_groups + g) * c.region_cells + tc] = make_double2(sa.value(), sb.value());
        }
    }
}

// One warp per packet: lanes are the packet's cells.
__global__ void adaptive_rays_kernel(const AdaptParams A) {
    const int lane = threadIdx.x & 31;
    const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarp = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long plane = (long long)A.na * A.nb;
    for (long long p = wid; p < A.n_packets; p += nwarp) {
        const int pa = (int)(p % A.npa);
        const long long rest = p / A.npa;
        const int pb = (int)(rest % A.npb), pw = (int)(rest / A.npb);
        const int jR = pa * A.tile_a + lane % A.tile_a, kR = pb * A.tile_b + lane / A.tile_a;
        float tsum = 0.0f, cnt = 0.0f;
        if (jR < A.njR && kR < A.nkR) {
            const int i = A.ew0 + pw;
            const float h = cbrtf((A.fw[i + 1] - A.fw[i]) * A.da * A.db);
            for (int f = 0; f < A.nfields; ++f) {
                const long long cell = f * A.field_stride + i * plane + (long long)(A.eb0 + kR) * A.na + (A.ea0 + jR);
                float kp = A.kappa;
                if (A.kP) {
                    int ti, xi = 0;
                    float ft, fx = 0.0f;
                    if (A.mode == MODE_TX) {
                        const float2 v = A.fTX[cell];
                        grid_pos(v.x, A.T0, A.invdT, A.nT, &ti, &ft);
                        grid_pos(v.y, A.X0, A.invdX, A.nX, &xi, &fx);
                    } else {
                        grid_pos(A.fT[cell], A.T0, A.invdT, A.nT, &ti, &ft);
                    }
                    const float *k = A.kP + ti * A.nX + xi;
                    const float dx = (A.nX > 1) ? 1.0f : 0.0f;
                    const float k00 = k[0], k01 = A.nX > 1 ? k[1] : k[0];
                    const float k10 = k[A.nX], k11 = A.nX > 1 ? k[A.nX + 1] : k[A.nX];
                    const float a0 = k00 + fx * dx * (k01 - k00), a1 = k10 + fx * dx * (k11 - k10);
                    kp = a0 + ft * (a1 - a0);
                }
                tsum += kp * h;
                cnt += 1.0f;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            tsum += __shfl_xor_sync(0xffffffffu, tsum, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) {
            const float x = A.per_tau * (cnt > 0.0f ? tsum / cnt : 0.0f);
            int r = (int)rintf(x / (float)A.B) * A.B;
            r = min(max(r, A.nmin), A.nmax);
            A.rays[p] = r;
        }
    }
}

int launch_adaptive_rays(const AdaptParams &a, void *stream) {
    const long long threads = (long long)a.n_packets * 32;
    adaptive_rays_kernel<<<grid_for(threads, 256), 256, 0, (cudaStream_t)stream>>>(a);
    return (int)cudaGetLastError();
}

int launch_cv_prepare(const CvParams &c, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    cv_layer_kernel<<<dim3(c.nw, c.nfields), 256, 0, st>>>(c);
    const long long n = (long long)c.nfields * c.n_samples * c.nw;
    cv_sur_kernel<<<grid_for(n, 256), 256, 0, st>>>(c);
    cv_jhat_kernel<<<grid_for(n, 128), 128, 0, st>>>(c);
    return (int)cudaGetLastError();
}

int launch_cv_mean(const CvParams &c, void *stream) {
    const long long n = (long long)c.nfields * c.region_cells;
    cv_mean_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(c);
    return (int)cudaGetLastError();
}

int march_occupancy(int mode, int threads) {
    int nb = 0;
    cudaError_t e = cudaErrorInvalidValue;
    if (mode == MODE_GREY) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_GREY, false, false>, threads, 0);
    if (mode == MODE_T) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_T, false, false>, threads, 0);
    if (mode == MODE_TX) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_kernel<MODE_TX, false, false>, threads, 0);
    if (e != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

int launch_field_pos(const float *fT, const float2 *fTX, float *outP, float2 *outPX, long long n, float T0,
                     float invdT, int nT, float X0, float invdX, int nX, void *stream) {
    field_pos_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(fT, fTX, outP, outPX, n, T0, invdT, nT,
                                                                        X0, invdX, nX);
    return (int)cudaGetLastError();
}

int launch_finalize(const FinalizeParams &p, void *stream) {
    const long long n = (long long)p.nfields * p.region_cells;
    finalize_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(p);
    return (int)cudaGetLastError();
}

int launch_pack_T(const float *src, float *dst, int nw, int na, int nb, long long si, long long sj,
                  long long sk, long long base, void *stream) {
    const long long n = (long long)nw * na * nb;
    pack_T_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(src, dst, nw, na, nb, si, sj, sk, base);
    return (int)cudaGetLastError();
}

int launch_pack_TX(const float *srcT, const float *srcX, float2 *dst, int nw, int na, int nb, long long si,
                   long long sj, long long sk, long long base, void *stream) {
    const long long n = (long long)nw * na * nb;
    pack_TX_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(srcT, srcX, dst, nw, na, nb, si, sj, sk, base);
    return (int)cudaGetLastError();
}

int launch_field_stats(const float *fT, const float2 *fTX, long long n, double *partials, float *out,
                       void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    field_stats_pass1<<<kStatBlocks, kStatThreads, 0, st>>>(fT, fTX, n, partials);
    field_stats_pass2<<<1, 32, 0, st>>>(partials, kStatBlocks, out);
    return (int)cudaGetLastError();
}

int field_stats_partials() { return 3 * kStatBlocks; }

int upload_sobol_dirs(const uint32_t dirs[4][32]) {
    return (int)cudaMemcpyToSymbol(c_sobol, dirs, sizeof(uint32_t) * 4 * 32);
}

int device_sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

}  // namespace dnsmc
