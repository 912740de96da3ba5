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
#include <atomic>

#include "mc_march.cuh"

namespace dnsmc {

// Table coordinates of the field for the march: p = clamp((T - T0)/dT, 0,
// nT-1) (and the same for x_H2O), computed once per solve with the same FP32
// operations the march used to apply per step.
__global__ void field_pos_kernel(const float *fT, const float2 *fTX, int2 *outP, int4 *outPX, long long n,
                                 float T0, float invdT, int nT, float X0, float invdX, int nX) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int ti, xi;
        float ft, fx;
        if (fTX) {
            const float2 v = fTX[i];
            float pt = (v.x - T0) * invdT;
            pt = fminf(fmaxf(pt, 0.0f), (float)(nT - 1));
            float px = (v.y - X0) * invdX;
            px = fminf(fmaxf(px, 0.0f), (float)(nX - 1));
            pos_split(pt, nT, &ti, &ft);
            pos_split(px, nX, &xi, &fx);
            outPX[i] = make_int4(ti * (nX - 1) + xi, __float_as_int(ft), __float_as_int(fx), ti);
        } else {
            float pt = (fT[i] - T0) * invdT;
            pt = fminf(fmaxf(pt, 0.0f), (float)(nT - 1));
            pos_split(pt, nT, &ti, &ft);
            outP[i] = make_int2(ti, __float_as_int(ft));
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
                // divisions by the ray counts as products with their
                // reciprocals (FP64 division is a long sequence on this GPU)
                const double2 r = F.rays_per_packet ? F.rcp[g * F.rays_gstride + p] : F.rcp_uniform;
                const long long ti = ((long long)f * F.n_groups + g) * F.region_cells + tc;
                const double2 t = F.tally[ti];
                m = t.x * r.x;
                if (F.batched) {
                    if (F.nbatch > 1) v = fmax(0.0, t.y * F.rcp_batch.x - m * m) * F.rcp_batch.y;
                } else if (N > 1) {
                    v = fmax(0.0, t.y * r.x - m * m) * r.y;
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
        if (F.sigma) F.sigma[idx] = sqrt(V);
        if (F.Qf) {  // the float results the host receives (8 bytes per cell)
            F.Qf[idx] = (float)Q;
            F.sigf[idx] = (float)sqrt(V * F.sig_scale);
        }
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
// Tmax, Tmin, sum of x and the count of temperatures that are not positive
// and finite, over n cells; two passes in a fixed order (deterministic).
__global__ void field_stats_pass1(const float *fT, const float2 *fTX, long long n, double *part) {
    __shared__ double smax[kStatThreads], smin[kStatThreads], ssum[kStatThreads], sbad[kStatThreads];
    double mx = -1e300, mn = 1e300, sm = 0.0, bad = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float T, x = 0.f;
        if (fTX) { const float2 v = fTX[i]; T = v.x; x = v.y; } else { T = fT[i]; }
        if (!(T > 0.0f) || !isfinite(T)) bad += 1.0;
        mx = fmax(mx, (double)T); mn = fmin(mn, (double)T); sm += x;
    }
    smax[threadIdx.x] = mx; smin[threadIdx.x] = mn; ssum[threadIdx.x] = sm; sbad[threadIdx.x] = bad;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
            sbad[threadIdx.x] += sbad[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double *p = part + 4 * blockIdx.x;
        p[0] = smax[0]; p[1] = smin[0]; p[2] = ssum[0]; p[3] = sbad[0];
    }
}
__global__ void field_stats_pass2(const double *part, int nparts, double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double mx = -1e300, mn = 1e300, sm = 0.0, bad = 0.0;
    for (int i = 0; i < nparts; ++i) {
        mx = fmax(mx, part[4 * i]); mn = fmin(mn, part[4 * i + 1]); sm += part[4 * i + 2]; bad += part[4 * i + 3];
    }
    out[0] = mx; out[1] = mn; out[2] = sm; out[3] = bad;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static std::atomic<long long> g_launches{0};
void note_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

static inline int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 4096) b = 4096;
    if (b < 1) b = 1;
    return (int)b;
}

int launch_march_ex(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                    bool mom, bool gen) {
    if (gen) return launch_march_gen(mode, p, blocks, threads, stream, trace, cv, mom);
    return launch_march_pair(mode, p, blocks, threads, stream, trace, cv, mom);
}

int march_occupancy_ex(int mode, int threads, bool cv, bool mom, bool gen, size_t smem) {
    if (gen) return march_gen_occupancy(mode, threads, cv, mom, smem);
    return march_pair_occupancy(mode, threads, cv, mom, smem);
}

// Multigrid march (reference tables or grey model; no control variate, no
// particles, black walls).
int launch_march_mg(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace) {
    cudaStream_t st = (cudaStream_t)stream;
    if (trace) { blocks = 1; threads = 32; }
    const size_t smem = march_smem(p, threads, 1);
    if (mode == MODE_GREY) {
        if (trace) return march_launch_one(march_mg_kernel<MODE_GREY, true>, blocks, threads,
                                           smem, st, p);
        return march_launch_one(march_mg_kernel<MODE_GREY, false>, blocks, threads, smem, st,
                                p);
    }
    if (mode == MODE_T) {
        if (trace) return march_launch_one(march_mg_kernel<MODE_T, true>, blocks, threads,
                                           smem, st, p);
        return march_launch_one(march_mg_kernel<MODE_T, false>, blocks, threads, smem, st, p);
    }
    return (int)cudaErrorInvalidValue;
}

int march_mg_occupancy(int mode, int threads, size_t smem) {
    int nb = 0;
    if (mode == MODE_GREY)
        nb = march_occupancy_one(march_mg_kernel<MODE_GREY, false>, threads, smem);
    if (mode == MODE_T) nb = march_occupancy_one(march_mg_kernel<MODE_T, false>, threads, smem);
    return nb > 0 ? nb : 1;
}

int launch_march(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace) {
    return launch_march_ex(mode, p, blocks, threads, stream, trace, false, false, false);
}

// ---------------------------------------------------------------------------
// Control variate preparation.  Y is the ray's contribution in the medium
// whose temperature and x_H2O are the mean of each wall-normal plane, with
// its flight through that medium replaced by a tabulated function of the
// ray's layer, spectral sample and wall-normal cosine mu:
//   J(mu) = the intensity the walk from the layer centre collects (same toll
//           cut-off, same wall emission as the 3-D march),
//   A(mu) = 1 - the transmissivity of its path out of the own layer,
// stored at the nodes u_m = m / kSurBins of u = sqrt(|mu|) per hemisphere and
// read by linear interpolation in u.  Whatever the table holds, its mean over
// the isotropic directions is a finite sum over the bins, so E[Y] per cell is
//   E[Y_a] = sum_s C_s k_i(s) (Ib_i(s) - Jhat_s(layer)),
//   E[Y_b] = sum_s C_s k_i(s) (Ib_i(s) - Ibar_s(layer)) Ahat_s(layer),
// exactly; the march tallies X - beta.Y and finalize adds beta.E[Y] back, so
// the estimate is unbiased for any beta and any table.
// ---------------------------------------------------------------------------
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
    __shared__ double sT[256], sX[256], sV[256];
    double aT = 0.0, aX = 0.0, aV = 0.0;
    for (long long i = threadIdx.x; i < plane; i += blockDim.x) {
        if (c.mode == MODE_TX) { const float2 v = c.fieldTX[base + i]; aT += v.x; aX += v.y; }
        else aT += c.fieldT[base + i];
        if (c.fieldV) aV += c.fieldV[base + i];
    }
    sT[threadIdx.x] = aT;
    sX[threadIdx.x] = aX;
    sV[threadIdx.x] = aV;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sT[threadIdx.x] += sT[threadIdx.x + o];
            sX[threadIdx.x] += sX[threadIdx.x + o];
            sV[threadIdx.x] += sV[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        c.layer[(long long)f * c.nw + w] = make_float2((float)(sT[0] / plane), (float)(sX[0] / plane));
        if (c.layerV) c.layerV[(long long)f * c.nw + w] = (float)(sV[0] / plane);
    }
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
        if (c.part) kb = fmaf(c.layerV[(long long)f * c.nw + w], c.part[c.mode == MODE_GREY ? 0 : sid / c.nq].x, kb);
        c.sur[idx] = make_float2(kb, Ib);
    }
}

// The straight walk of the surrogate: from oW (the centre of layer w0) with
// wall-normal cosine mu > 0 in direction dW (+1: east), through the layers of
// constant (k, Ib) = surp[l], advanced layer by layer and stopped when its
// optical depth exceeds dtoll = ln(1/toll) (the rest is absorbed in that
// layer) or at the black wall of intensity Iw.  Returns the collected
// intensity J and the own-layer absorptance A = 1 - (transmissivity leaving
// layer w0; 0 if the walk stops inside it).
__device__ __forceinline__ void cv_walk(const float *fw, int nw, float dtoll, const float2 *surp, int w0, float oW,
                                        float mu, int dW, float Iw, float *J_out, float *A_out) {
    const float invW = 1.0f / mu;
    // exit face of layer l at parameter (fw[l + 1] - o)/mu going east and
    // (fw[l] - o) * (-1/mu) going west
    const float *fwn = fw + (dW > 0 ? 1 : 0);
    const float sinvW = dW > 0 ? invW : -invW;
    const int lwall = dW > 0 ? nw : -1;
    float J = 0.0f, tauE = 1.0f, tE = 0.0f, dcum = 0.0f, tex0 = -1.0f;
    int l = w0;
    float2 kv = __ldg(surp + w0);
    bool trunc;
    for (;;) {
        const float tn = (__ldg(fwn + l) - oW) * sinvW;
        const float opt = kv.x * (tn - tE);
        trunc = dcum + opt > dtoll;
        if (trunc) break;  // truncated in layer l
        const float as = -mc_expm1(-opt);
        const float tas = tauE * as;
        J = fmaf(tas, kv.y, J);
        tauE = tauE - tas;
        dcum = dcum + opt;
        tE = tn;
        tex0 = tex0 < 0.0f ? tauE : tex0;
        l += dW;
        if (l == lwall) break;  // reached the wall
        kv = __ldg(surp + l);
    }
    *J_out = fmaf(tauE, trunc ? kv.y : Iw, J);
    *A_out = 1.0f - (tex0 < 0.0f ? 0.0f : tex0);
}

// Surrogate table and its exact means per (field, sample, layer), one warp
// each: the lanes walk the 2 (kSurBins + 1) nodes (mu = u_m^2, u_m = m /
// kSurBins; the node u = 0 at mu = 2^-30, the grazing limit), the warp's
// shared row holds them, and each lane writes kSurBins / 16 bins and their
// FP64 contribution to the means.  With mu uniform on [0, 1] per hemisphere,
// u has density 2u, and a bin m contributes
//   E_h[J] += ((2m + 1) J0 + (m + 2/3) dJ) / kSurBins^2,
// likewise for A; the warp sums in butterfly order.
constexpr int kSurNodes = kSurBins + 1;
__global__ void cv_table_kernel(const CvParams c) {
    __shared__ float2 s_node[8][2 * kSurNodes];
    const long long n = (long long)c.nfields * c.n_samples * c.nw;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long wpb = blockDim.x >> 5;
    float2 *node = s_node[wid];
    for (long long idx = blockIdx.x * wpb + wid; idx < n; idx += (long long)gridDim.x * wpb) {
        const int w = (int)(idx % c.nw);
        const long long fs = idx / c.nw;
        const int sid = (int)(fs % c.n_samples);
        const float2 *sp = c.sur + fs * c.nw;
        const int band = c.mode == MODE_GREY ? 0 : sid / c.nq;
        const float oW = (__ldg(c.fw + w) + __ldg(c.fw + w + 1)) * 0.5f;
        for (int e = lane; e < 2 * kSurNodes; e += 32) {
            const int h = e >= kSurNodes ? 1 : 0;
            const int m = e - h * kSurNodes;
            const float u = (float)m * (1.0f / (float)kSurBins);
            const float mu = m ? u * u : 9.31322574615478516e-10f;  // 2^-30
            const float Iw = c.mode == MODE_GREY ? c.Tw4[h] : __ldg(c.ibw + h * c.nbands + band);
            float J, A;
            cv_walk(c.fw, c.nw, c.dtoll, sp, w, oW, mu, h ? 1 : -1, Iw, &J, &A);
            node[e] = make_float2(J, A);
        }
        __syncwarp();
        float4 *row = c.surtab + idx * (2 * kSurBins);
        double eJ = 0.0, eA = 0.0;
#pragma unroll
        for (int j = 0; j < (2 * kSurBins) / 32; ++j) {
            const int bi = lane + 32 * j;
            const int h = bi >= kSurBins ? 1 : 0;
            const int m = bi - h * kSurBins;
            const float2 v0 = node[h * kSurNodes + m], v1 = node[h * kSurNodes + m + 1];
            const float dJ = v1.x - v0.x, dA = v1.y - v0.y;
            row[bi] = make_float4(v0.x, dJ, v0.y, dA);
            const double c0 = (double)(2 * m + 1), c1 = (double)m + 2.0 / 3.0;
            eJ += c0 * (double)v0.x + c1 * (double)dJ;
            eA += c0 * (double)v0.y + c1 * (double)dA;
        }
        for (int o = 16; o > 0; o >>= 1) {
            eJ += __shfl_xor_sync(0xffffffffu, eJ, o);
            eA += __shfl_xor_sync(0xffffffffu, eA, o);
        }
        if (lane == 0) {
            const double sc = 0.5 / ((double)kSurBins * (double)kSurBins);  // both hemispheres, weight 1/2
            const double J = eJ * sc, A = eA * sc;
            const float Jhi = (float)J;
            c.Jhat[idx] = make_double2(J, A);
            c.Jf[idx] = make_float4(Jhi, (float)(J - (double)Jhi), (float)A, sp[w].y);
        }
        __syncwarp();
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
        const float fv = c.fieldV ? c.fieldV[cell] : 0.0f;
        if (c.mode == MODE_GREY) {
            const float t2 = T * T;
            const double2 jh = c.Jhat[sbase];
            // the march's own FP32 weight 4 sigma (kappa + fv a) when particles are present
            const double Wk = c.part ? (double)((float)(4.0 * 5.670373e-08) * fmaf(fv, c.part[0].x, c.kappa)) : c.Wgrey;
            const double acc = Wk * ((double)(t2 * t2) - jh.x);
            const double accB = Wk * ((double)(t2 * t2) - (double)c.sur[sbase].y) * jh.y;
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
                if (c.part) k = fmaf(fv, __ldg(&c.part[sid / c.nq].x), k);
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

// ---------------------------------------------------------------------------
// E[Y] through node sums (tables without particles).  With k_s(T, x) the
// bilinear and Ib_s(T) the linear interpolant of the tables at the cell's
// table coordinates (weights wt_a in T, wx_b in x),
//   E[Y_a] = sum_s C_s k_s Ib_s - sum_s C_s Jhat_s(w) k_s,
//   E[Y_b] = sum_s C_s Ahat_s(w) k_s Ib_s - sum_s C_s Ahat_s(w) Ibar_s(w) k_s,
// and every sum is a fixed combination of sums over the samples taken at
// the table nodes:
//   GJ(w)[t][x]          = sum_s C_s Jhat_s(w) k_s[t][x]
//   GB(w)[t][x]          = sum_s C_s Ahat_s(w) Ibar_s(w) k_s[t][x]
//   MB(w)[t][x][a][a']   = sum_s C_s Ahat_s(w) k_s[t+a][x] Ib_s[t+a']
//   M[t][x][a][a']       = sum_s C_s k_s[t+a][x] Ib_s[t+a']      (no layer)
// so a cell needs 24 node sums per group instead of a pass over the group's
// samples.  FP64 throughout (sums over the samples, and the cell's
// combination): exact to the FP32 rounding of the march's own lookups.
// ---------------------------------------------------------------------------
struct NodeLayout {
    int nTX, nM, per;  // nodes, (t cell, x node, a, a') entries, doubles per (field, group, layer)
};
__host__ __device__ inline NodeLayout node_layout(const CvParams &c) {
    NodeLayout L;
    L.nTX = c.nT * c.nX;
    L.nM = (c.nT - 1) * c.nX * 4;
    L.per = 2 * L.nTX + L.nM;
    return L;
}

long long cv_node_count(const CvParams &c) {
    const NodeLayout L = node_layout(c);
    const long long niR = c.ew1 - c.ew0;
    return (long long)c.nfields * c.n_groups * niR * L.per + (long long)c.n_groups * L.nM;
}

// Blocks: (field, group, region layer), then one per group for M.  Work
// units of a block: the nodes of GJ and of GB (one sum each), and the table
// cells (t, x) of MB or M (the four sums over a, a' together).  The tables
// are read as FP64 copies, the per-sample weights come from shared memory,
// so a sum costs one FP64 fma per sample (1.5 for MB / M).
__global__ void cv_nodes_kernel(const CvParams c) {
    __shared__ int s_band[256];
    __shared__ int s_koff[256];
    __shared__ double s_wJ[256], s_wB[256], s_wM[256];
    const NodeLayout L = node_layout(c);
    const int niR = c.ew1 - c.ew0;
    const int nTc = c.nT - 1;  // table cells along T
    const long long nlay = (long long)c.nfields * c.n_groups * niR;
    const long long b = blockIdx.x;
    const bool layered = b < nlay;
    int f = 0, g, w = 0;
    double *out;
    if (layered) {
        const int wR = (int)(b % niR);
        const long long fg = b / niR;
        g = (int)(fg % c.n_groups);
        f = (int)(fg / c.n_groups);
        w = c.ew0 + wR;
        out = c.nodes + b * L.per;
    } else {
        g = (int)(b - nlay);
        out = c.nodes + nlay * L.per + (long long)g * L.nM;
    }
    // units: [GJ nodes | GB nodes] (layered only), then (t, x) table cells
    const int nnode = layered ? 2 * L.nTX : 0;
    const int nunit = nnode + nTc * c.nX;
    const int q0 = c.grp_start[g], q1 = c.grp_start[g + 1];
    constexpr int kMaxUnits = 8;
    double acc[kMaxUnits][4];
#pragma unroll
    for (int i = 0; i < kMaxUnits; ++i)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[i][r] = 0.0;
    for (int qc = q0; qc < q1; qc += 256) {
        const int nq = min(256, q1 - qc);
        __syncthreads();
        if ((int)threadIdx.x < nq) {
            const int q = qc + threadIdx.x;
            const int sid = c.samp_id[q];
            const double C = c.samp_C[q];
            s_band[threadIdx.x] = (sid / c.nq) * c.nT;
            s_koff[threadIdx.x] = sid * c.nT * c.nX;
            if (layered) {
                const long long o = ((long long)f * c.n_samples + sid) * c.nw + w;
                const double2 jh = c.Jhat[o];
                s_wJ[threadIdx.x] = C * jh.x;
                s_wB[threadIdx.x] = C * jh.y * (double)c.sur[o].y;
                s_wM[threadIdx.x] = C * jh.y;
            } else {
                s_wM[threadIdx.x] = C;
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kMaxUnits; ++i) {
            const int u = threadIdx.x + i * blockDim.x;
            if (u >= nunit) break;
            if (u < nnode) {  // GJ or GB at node n
                const bool gb = u >= L.nTX;
                const int n = gb ? u - L.nTX : u;
                const double *wv = gb ? s_wB : s_wJ;
                double sum = acc[i][0];
                for (int j = 0; j < nq; ++j) sum = fma(wv[j], __ldg(c.ktab_d + s_koff[j] + n), sum);
                acc[i][0] = sum;
            } else {  // table cell (t, x): sums over a, a' of k[t+a][x] Ib[t+a']
                const int m = u - nnode;
                const int t = m / c.nX, x = m - t * c.nX;
                double s00 = acc[i][0], s01 = acc[i][1], s10 = acc[i][2], s11 = acc[i][3];
                for (int j = 0; j < nq; ++j) {
                    const double *kk = c.ktab_d + s_koff[j] + t * c.nX + x;
                    const double *ib = c.ibtab_d + s_band[j] + t;
                    const double k0 = s_wM[j] * __ldg(kk), k1 = s_wM[j] * __ldg(kk + c.nX);
                    const double i0 = __ldg(ib), i1 = __ldg(ib + 1);
                    s00 = fma(k0, i0, s00);
                    s01 = fma(k0, i1, s01);
                    s10 = fma(k1, i0, s10);
                    s11 = fma(k1, i1, s11);
                }
                acc[i][0] = s00; acc[i][1] = s01; acc[i][2] = s10; acc[i][3] = s11;
            }
        }
    }
    // layout: GJ [nTX], GB [nTX], then MB / M [t][x][a*2 + a']
    double *mout = out + (layered ? 2 * L.nTX : 0);
#pragma unroll
    for (int i = 0; i < kMaxUnits; ++i) {
        const int u = threadIdx.x + i * blockDim.x;
        if (u >= nunit) break;
        if (u < nnode) {
            out[u] = acc[i][0];
        } else {
            double *o = mout + (long long)(u - nnode) * 4;
            o[0] = acc[i][0]; o[1] = acc[i][1]; o[2] = acc[i][2]; o[3] = acc[i][3];
        }
    }
}

// E[Y] per (field, cell) from the node sums, all groups.
__global__ void cv_mean_nodes_kernel(const CvParams c) {
    const NodeLayout L = node_layout(c);
    const int njR = c.ea1 - c.ea0, nkR = c.eb1 - c.eb0, niR = c.ew1 - c.ew0;
    const long long n = (long long)c.nfields * c.region_cells;
    const long long plane = (long long)c.na * c.nb;
    const double *M = c.nodes + (long long)c.nfields * c.n_groups * niR * L.per;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(idx / c.region_cells);
        const long long tc = idx - (long long)f * c.region_cells;
        const int jR = (int)(tc % njR);
        const long long r = tc / njR;
        const int kR = (int)(r % nkR);
        const int iR = (int)(r / nkR);
        const long long cell = (long long)f * c.nw * plane + (long long)(c.ew0 + iR) * plane +
                               (long long)(c.eb0 + kR) * c.na + (c.ea0 + jR);
        float T, x = 0.f;
        if (c.mode == MODE_TX) { const float2 v = c.fieldTX[cell]; T = v.x; x = v.y; }
        else T = c.fieldT[cell];
        int ti, xi = 0;
        float ftf, fxf = 0.f;
        grid_pos(T, c.T0, c.invdT, c.nT, &ti, &ftf);
        if (c.mode == MODE_TX) grid_pos(x, c.X0, c.invdX, c.nX, &xi, &fxf);
        const double ft = ftf, fx = fxf;
        const double wt[2] = {1.0 - ft, ft};
        const double wx[2] = {1.0 - fx, fx};
        const int nb = c.nX > 1 ? 2 : 1;
        // the cell's interpolation weights, formed once for all groups:
        // w4[bx][a][a'] = wx[bx] wt[a] wt[a'] (the product of the k and Ib
        // interpolations) and w2[bx][a] = wx[bx] wt[a]
        double w4[2][4], w2[2][2];
        for (int bx = 0; bx < nb; ++bx)
            for (int a = 0; a < 2; ++a) {
                w2[bx][a] = wx[bx] * wt[a];
                for (int a2 = 0; a2 < 2; ++a2) w4[bx][a * 2 + a2] = w2[bx][a] * wt[a2];
            }
        for (int g = 0; g < c.n_groups; ++g) {
            const double *lay = c.nodes + (((long long)f * c.n_groups + g) * niR + iR) * L.per;
            const double *GJ = lay, *GB = lay + L.nTX, *MB = lay + 2 * L.nTX;
            const double *Mg = M + (long long)g * L.nM;
            double kI = 0.0, kJ = 0.0, kIA = 0.0, kB = 0.0;
            for (int bx = 0; bx < nb; ++bx) {
                const int xn = xi + bx;
                const double *m = Mg + ((long long)ti * c.nX + xn) * 4;
                const double *mb = MB + ((long long)ti * c.nX + xn) * 4;
                for (int q = 0; q < 4; ++q) {
                    kI = fma(w4[bx][q], m[q], kI);
                    kIA = fma(w4[bx][q], mb[q], kIA);
                }
                for (int a = 0; a < 2; ++a) {
                    kJ = fma(w2[bx][a], GJ[(ti + a) * c.nX + xn], kJ);
                    kB = fma(w2[bx][a], GB[(ti + a) * c.nX + xn], kB);
                }
            }
            c.muY[((long long)f * c.n_groups + g) * c.region_cells + tc] = make_double2(kI - kJ, kIA - kB);
        }
    }
}

// One warp per packet: lane l takes the packet's cells l, l + 32, ...
__global__ void adaptive_rays_kernel(const AdaptParams A) {
    const int lane = threadIdx.x & 31;
    const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarp = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long plane = (long long)A.na * A.nb;
    for (long long p = wid; p < A.n_packets; p += nwarp) {
        const int pa = (int)(p % A.npa);
        const long long rest = p / A.npa;
        const int pb = (int)(rest % A.npb), pw = (int)(rest / A.npb);
        float tsum = 0.0f, cnt = 0.0f;
        for (int cl = lane; cl < A.tile_a * A.tile_b; cl += 32) {
            const int jR = pa * A.tile_a + cl % A.tile_a, kR = pb * A.tile_b + cl / A.tile_a;
            if (jR >= A.njR || kR >= A.nkR) continue;
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
    dnsmc::note_launch();
    adaptive_rays_kernel<<<grid_for(threads, 256), 256, 0, (cudaStream_t)stream>>>(a);
    return (int)cudaGetLastError();
}

// Longest-first queue order.  Bucket of an item = min(rays / B, buckets - 1),
// counted in descending bucket order; items of one bucket keep no particular
// order (results do not depend on the processing order).
__global__ void order_hist_kernel(const int *rays, int gstride, int n_packets, int n_groups, long long n_items, int B,
                                  unsigned int *hist) {
    const long long per_field = (long long)n_groups * n_packets;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_items;
         i += (long long)gridDim.x * blockDim.x) {
        const long long gp = i % per_field;
        const int g = (int)(gp / n_packets), p = (int)(gp % n_packets);
        const int b = min(rays[g * gstride + p] / B, kOrderBuckets - 1);
        atomicAdd(hist + (kOrderBuckets - 1 - b), 1u);
    }
}

// exclusive scan of the kOrderBuckets counts in place (one block of 1024)
__global__ void order_scan_kernel(unsigned int *hist) {
    __shared__ unsigned int part[1024];
    constexpr int per = kOrderBuckets / 1024;
    const int t = threadIdx.x;
    unsigned int loc[per], run = 0;
    for (int q = 0; q < per; ++q) { loc[q] = hist[t * per + q]; run += loc[q]; }
    part[t] = run;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned int v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    unsigned int base = t ? part[t - 1] : 0u;
    for (int q = 0; q < per; ++q) { const unsigned int v = loc[q]; hist[t * per + q] = base; base += v; }
}

__global__ void order_scatter_kernel(const int *rays, int gstride, int n_packets, int n_groups, long long n_items,
                                     int B, unsigned int *hist, unsigned int *order) {
    const long long per_field = (long long)n_groups * n_packets;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_items;
         i += (long long)gridDim.x * blockDim.x) {
        const long long gp = i % per_field;
        const int g = (int)(gp / n_packets), p = (int)(gp % n_packets);
        const int b = min(rays[g * gstride + p] / B, kOrderBuckets - 1);
        const unsigned int pos = atomicAdd(hist + (kOrderBuckets - 1 - b), 1u);
        order[pos] = (unsigned int)i;
    }
}

int launch_item_order(const int *rays, int gstride, int n_packets, int n_groups, long long n_items, int B,
                      unsigned int *hist, unsigned int *order, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(hist, 0, kOrderBuckets * sizeof(unsigned int), st);
    if (e != cudaSuccess) return (int)e;
    dnsmc::note_launch();
    order_hist_kernel<<<grid_for(n_items, 256), 256, 0, st>>>(rays, gstride, n_packets, n_groups, n_items, B, hist);
    dnsmc::note_launch();
    order_scan_kernel<<<1, 1024, 0, st>>>(hist);
    dnsmc::note_launch();
    order_scatter_kernel<<<grid_for(n_items, 256), 256, 0, st>>>(rays, gstride, n_packets, n_groups, n_items, B,
                                                                 hist, order);
    return (int)cudaGetLastError();
}

int launch_cv_prepare(const CvParams &c, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    dnsmc::note_launch();
    cv_layer_kernel<<<dim3(c.nw, c.nfields), 256, 0, st>>>(c);
    const long long n = (long long)c.nfields * c.n_samples * c.nw;
    dnsmc::note_launch();
    cv_sur_kernel<<<grid_for(n, 256), 256, 0, st>>>(c);
    dnsmc::note_launch();
    cv_table_kernel<<<grid_for(n * 32, 256), 256, 0, st>>>(c);  // one warp per (field, sample, layer)
    return (int)cudaGetLastError();
}

int launch_cv_mean(const CvParams &c, void *stream) {
    const long long n = (long long)c.nfields * c.region_cells;
    cudaStream_t st = (cudaStream_t)stream;
    if (c.nodes) {  // tables without particles: node sums, then the cells
        const long long blocks = (long long)c.nfields * c.n_groups * (c.ew1 - c.ew0) + c.n_groups;
        dnsmc::note_launch();
        cv_nodes_kernel<<<(unsigned)blocks, 256, 0, st>>>(c);
        dnsmc::note_launch();
        cv_mean_nodes_kernel<<<grid_for(n, 256), 256, 0, st>>>(c);
    } else {
        dnsmc::note_launch();
        cv_mean_kernel<<<grid_for(n, 256), 256, 0, st>>>(c);
    }
    return (int)cudaGetLastError();
}

int march_occupancy(int mode, int threads) { return march_occupancy_ex(mode, threads, false, false, false, 0); }

int launch_field_pos(const float *fT, const float2 *fTX, int2 *outP, int4 *outPX, long long n, float T0,
                     float invdT, int nT, float X0, float invdX, int nX, void *stream) {
    dnsmc::note_launch();
    field_pos_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(fT, fTX, outP, outPX, n, T0, invdT, nT,
                                                                        X0, invdX, nX);
    return (int)cudaGetLastError();
}

// (1/N, 1/(N-1)) of every ray count (0 where undefined)
__global__ void ray_reciprocals_kernel(const int *rays, long long n, double2 *out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int N = rays[i];
        out[i] = make_double2(N > 0 ? 1.0 / N : 0.0, N > 1 ? 1.0 / (N - 1) : 0.0);
    }
}

static double2 reciprocals(int N) { return make_double2(N > 0 ? 1.0 / N : 0.0, N > 1 ? 1.0 / (N - 1) : 0.0); }

int launch_finalize(const FinalizeParams &p, void *stream) {
    FinalizeParams q = p;
    q.rcp_uniform = reciprocals(p.rays);
    q.rcp_batch = reciprocals(p.nbatch);
    cudaStream_t st = (cudaStream_t)stream;
    if (q.rays_per_packet) {
        if (!q.rcp) return (int)cudaErrorInvalidValue;
        const long long nr = finalize_rcp_count(q);
        dnsmc::note_launch();
        ray_reciprocals_kernel<<<grid_for(nr, 256), 256, 0, st>>>(q.rays_per_packet, nr, q.rcp);
    }
    const long long n = (long long)q.nfields * q.region_cells;
    dnsmc::note_launch();
    finalize_kernel<<<grid_for(n, 256), 256, 0, st>>>(q);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Spline coarsening of the temperature for the multigrid march: the
// reference's interp3D (code/spline.cpp:35-116), a separable natural cubic
// spline through the fine cell centres along x, then y, then z, evaluated at
// the coarse cell centres.  One thread per spline line; each pass is one
// launch.  The arithmetic is the Numerical Recipes spline / splint of
// code/spline.cpp:119-170 written as the oracle restates it (float with the
// same double sub-expressions; this translation unit is compiled with
// -fmad=false), so the coarse fields are bit-identical to the oracle's.
// ---------------------------------------------------------------------------
__global__ void spline_pass_kernel(SplinePass q) {
    for (long long L = blockIdx.x * (long long)blockDim.x + threadIdx.x; L < q.nlines;
         L += (long long)gridDim.x * blockDim.x) {
        const long long la = L % q.na, lb = L / q.na;
        const float *src = q.src + (la * q.s_a + lb * q.s_b) * q.src_step;
        float *dst = q.dst + la * q.d_a + lb * q.d_b;
        // this line's work arrays, interleaved across lines (1-based, n + 2)
        float *a = q.work + L;
        float *y2 = a + (long long)(q.n + 2) * q.nlines;
        float *u = y2 + (long long)(q.n + 2) * q.nlines;
        const long long w = q.nlines;
        const float *x = q.xf;
        const int n = q.n;
        for (int i = 1; i <= n; ++i) a[i * w] = src[(long long)(i - 1) * q.s_e * q.src_step];
        // second derivatives (natural end conditions)
        y2[1 * w] = 0.0f;
        u[1 * w] = 0.0f;
        for (int i = 2; i <= n - 1; ++i) {
            const float sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
            const float p = sig * y2[(i - 1) * w] + 2.0f;
            y2[i * w] = (sig - 1.0f) / p;
            const float ui = (a[(i + 1) * w] - a[i * w]) / (x[i + 1] - x[i]) -
                             (a[i * w] - a[(i - 1) * w]) / (x[i] - x[i - 1]);
            u[i * w] = (float)((6.0 * ui / (x[i + 1] - x[i - 1]) - sig * u[(i - 1) * w]) / p);
        }
        y2[n * w] = 0.0f;
        for (int k = n - 1; k >= 1; --k) y2[k * w] = y2[k * w] * y2[(k + 1) * w] + u[k * w];
        // values at the coarse centres (bisection for the bracket)
        for (int c = 1; c <= q.m; ++c) {
            const float v = q.xc[c];
            int lo = 1, hi = n;
            while (hi - lo > 1) {
                const int k = (hi + lo) >> 1;
                if (x[k] > v) hi = k; else lo = k;
            }
            const float h = x[hi] - x[lo];
            const float aa = (x[hi] - v) / h, bb = (v - x[lo]) / h;
            const float ylo = a[lo * w], yhi = a[hi * w];
            dst[(long long)(c - 1) * q.d_e] =
                (float)(aa * ylo + bb * yhi +
                        ((aa * aa * aa - aa) * y2[lo * w] + (bb * bb * bb - bb) * y2[hi * w]) * (h * h) / 6.0);
        }
    }
}

int launch_spline_pass(const SplinePass &q, void *stream) {
    if (q.nlines <= 0) return 0;
    dnsmc::note_launch();
    spline_pass_kernel<<<grid_for(q.nlines, 128), 128, 0, (cudaStream_t)stream>>>(q);
    return (int)cudaGetLastError();
}

int launch_pack_T(const float *src, float *dst, int nw, int na, int nb, long long si, long long sj,
                  long long sk, long long base, void *stream) {
    const long long n = (long long)nw * na * nb;
    dnsmc::note_launch();
    pack_T_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(src, dst, nw, na, nb, si, sj, sk, base);
    return (int)cudaGetLastError();
}

int launch_pack_TX(const float *srcT, const float *srcX, float2 *dst, int nw, int na, int nb, long long si,
                   long long sj, long long sk, long long base, void *stream) {
    const long long n = (long long)nw * na * nb;
    dnsmc::note_launch();
    pack_TX_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(srcT, srcX, dst, nw, na, nb, si, sj, sk, base);
    return (int)cudaGetLastError();
}

int launch_field_stats(const float *fT, const float2 *fTX, long long n, double *partials, double *out,
                       void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    dnsmc::note_launch();
    field_stats_pass1<<<kStatBlocks, kStatThreads, 0, st>>>(fT, fTX, n, partials);
    dnsmc::note_launch();
    field_stats_pass2<<<1, 32, 0, st>>>(partials, kStatBlocks, out);
    return (int)cudaGetLastError();
}

int field_stats_partials() { return 4 * kStatBlocks; }

int upload_sobol_dirs(const uint32_t dirs[4][32]) {
    int rc = (int)cudaMemcpyToSymbol(c_sobol, dirs, sizeof(uint32_t) * 4 * 32);
    if (rc) return rc;
    rc = upload_sobol_dirs_gen(dirs);
    return rc ? rc : upload_sobol_dirs_pair(dirs);
}

int device_sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

}  // namespace dnsmc
