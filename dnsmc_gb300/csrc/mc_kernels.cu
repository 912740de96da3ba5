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
// One block per tile of 32 j x 32 i cells of a k row of a field: the tally
// layout has j fastest and the outputs i fastest, so the block reads its
// cells along j (thread x = j) and writes them along i through a
// shared-memory transpose.  Every cell's arithmetic is in the same order as
// a plain per-cell loop over the groups.
constexpr int kFinTile = 32, kFinRows = 8;
__global__ void __launch_bounds__(kFinTile * kFinRows) finalize_kernel(const FinalizeParams F) {
    __shared__ double s_a[kFinTile][kFinTile + 1], s_b[kFinTile][kFinTile + 1];  // [i][j]
    const int tx = threadIdx.x % kFinTile, ty = threadIdx.x / kFinTile;
    const int ntj = (F.njR + kFinTile - 1) / kFinTile;
    const int j0 = (blockIdx.x % ntj) * kFinTile, i0 = (blockIdx.x / ntj) * kFinTile;
    const int kR = blockIdx.y, f = blockIdx.z;
    constexpr int S = kFinTile / kFinRows;  // cells per thread
    // read side: cell s of this thread is (iR = i0 + ty + kFinRows s, jR = j0 + tx)
    const int jR = j0 + tx;
    double Q[S], V[S];
#pragma unroll
    for (int s = 0; s < S; ++s) { Q[s] = 0.0; V[s] = 0.0; }
    // write side: thread x = i, cell s at (iR = i0 + tx, jR = j0 + ty + kFinRows s)
    const int iW = i0 + tx;
    for (int g = 0; g < F.n_groups; ++g) {
        double mg[S], vg[S];
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const int iR = i0 + ty + kFinRows * s;
            double m = 0.0, v = 0.0;
            if (iR < F.niR && jR < F.njR) {
                const long long tc = ((long long)iR * F.nkR + kR) * F.njR + jR;
                const int p = (iR * F.npb + kR / F.tile_b) * F.npa + jR / F.tile_a;
                const int N = F.rays_per_packet ? F.rays_per_packet[g * F.rays_gstride + p] : F.rays;
                const long long ti = ((long long)f * F.n_groups + g) * F.region_cells + tc;
                if (!F.group_empty[g] && N > 0) {
                    // divisions by the ray counts as products with their
                    // reciprocals (FP64 division is a long sequence on this GPU)
                    const double2 r = F.rays_per_packet ? F.rcp[g * F.rays_gstride + p] : F.rcp_uniform;
                    const double2 t = F.tally[ti];
                    m = t.x * r.x;
                    if (F.batched) {
                        if (F.nbatch > 1) v = fmax(0.0, t.y * F.rcp_batch.x - m * m) * F.rcp_batch.y;
                    } else if (N > 1) {
                        v = fmax(0.0, t.y * r.x - m * m) * r.y;
                    }
                }
                if (F.muY && !F.group_empty[g]) {
                    const float2 b = F.beta ? F.beta[ti] : make_float2(1.0f, -1.0f);
                    const double2 mu = F.muY[ti];
                    // Q_g = beta_a E[Y_a] + beta_b E[Y_b] + mean(X - beta_a Y_a - beta_b Y_b)
                    m += (double)b.x * mu.x;
                    m += (double)b.y * mu.y;
                }
            }
            Q[s] += m;
            V[s] += v;
            mg[s] = m;
            vg[s] = v;
        }
        if (F.Qg) {  // the group's results, [f][group][cell] i fastest
#pragma unroll
            for (int s = 0; s < S; ++s) { s_a[ty + kFinRows * s][tx] = mg[s]; s_b[ty + kFinRows * s][tx] = vg[s]; }
            __syncthreads();
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const int jW = j0 + ty + kFinRows * s;
                if (iW < F.niR && jW < F.njR) {
                    const long long o = ((long long)f * F.n_groups + g) * F.region_cells +
                                        ((long long)kR * F.njR + jW) * F.niR + iW;
                    F.Qg[o] = s_a[tx][ty + kFinRows * s];
                    F.varg[o] = s_b[tx][ty + kFinRows * s];
                }
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int s = 0; s < S; ++s) { s_a[ty + kFinRows * s][tx] = Q[s]; s_b[ty + kFinRows * s][tx] = V[s]; }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int jW = j0 + ty + kFinRows * s;
        if (iW < F.niR && jW < F.njR) {
            const double Qc = s_a[tx][ty + kFinRows * s], Vc = s_b[tx][ty + kFinRows * s];
            const long long idx = (long long)f * F.region_cells + ((long long)kR * F.njR + jW) * F.niR + iW;
            F.Q[idx] = Qc;
            F.var[idx] = Vc;
            const double sd = sqrt(Vc);
            if (F.sigma) F.sigma[idx] = sd;
            if (F.Qf) {  // the float results the host receives (8 bytes per cell)
                F.Qf[idx] = (float)Qc;
                // one FP64 square root per cell when no scale applies
                F.sigf[idx] = (float)(F.sig_scale == 1.0 ? sd : sqrt(Vc * F.sig_scale));
            }
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

// Surrogate table and its exact means, one block per (field, sample).  The
// surrogate ray leaves the centre o_l of layer l with wall-normal cosine mu
// and flies straight through the layers of constant (k, Ib) = sur[l] to the
// black wall (intensity Iw); what it collects is
//   J_l = (1 - e^{-h_l}) Ib_l + e^{-h_l} F_{l+1}   (east; west alike),
// with h_l = k_l (f_{l+1} - o_l) / mu its own half-layer depth and F_i the
// intensity collected by a ray entering layer i from the west face,
//   F_i = (1 - e^{-d_i}) Ib_i + e^{-d_i} F_{i+1},  F_nw = Iw,  d_i = k_i (f_{i+1} - f_i) / mu,
// and its own-layer absorptance is A_l = 1 - e^{-h_l}.  So one sweep per
// (node, hemisphere) from the far wall gives every layer's node: thread
// (h, m) sweeps mu = u_m^2 (u_m = m / kSurBins; the node u = 0 at mu =
// 2^-30, the grazing limit) across the layers, one layer per step, with
// e^{-x} - 1 = mc_expm1(-x):
//   J = F + e1h (F - Ib_l),  A = -e1h,  then  F <- F + e1 (F - Ib_l).
// After each step the block writes the two layers' bins (J0, dJ, A0, dA)
// and their contributions to the means: with mu uniform on [0, 1] per
// hemisphere, u has density 2u, and bin m contributes
//   E_h[J] += ((2m + 1) J0 + (m + 2/3) dJ) / kSurBins^2
//          = (3 (2m + 1) J0 + (3m + 2) dJ) / (3 kSurBins^2),
// likewise for A.  The integer-weighted terms are formed exactly as
// float pairs (the product's rounding error by fma) and summed as float
// pairs (error-free sums), each hemisphere's 64 terms by two warps in
// butterfly order, then in FP64: about 48 bits, at FP32 rates (this GPU's
// FP64 rate is a small fraction of that).
constexpr int kSurNodes = kSurBins + 1;

// (hi, lo) float pairs: ff_add (mc_march.cuh) sums two of them
// w * v as an exact pair (w a small integer)
__device__ __forceinline__ float2 ff_mul(float w, float v) {
    const float p = w * v;
    return make_float2(p, fmaf(w, v, -p));
}
constexpr int kTableThreads = 160;  // 2 kSurNodes sweeps; 2 kSurBins bins
size_t cv_table_smem(int nw) { return (size_t)nw * (2 * sizeof(double2) + sizeof(float2) + sizeof(float)) + 16; }

__global__ void __launch_bounds__(kTableThreads) cv_table_kernel(const CvParams c) {
    extern __shared__ double2 s_mean[];                    // [nw][2] per-hemisphere sums (eJ, eA)
    float2 *s_sur = reinterpret_cast<float2 *>(s_mean + 2 * c.nw);  // [nw] (k, Ib)
    float *s_fw = reinterpret_cast<float *>(s_sur + c.nw);  // [nw + 1] faces
    __shared__ float2 s_val[2][kSurNodes];                 // this step's nodes (J, A)
    __shared__ double2 s_half[4];                          // this step's warp sums
    const int t = threadIdx.x, nw = c.nw;
    const long long fs = blockIdx.x;                       // field * n_samples + sample
    const int sid = (int)(fs % c.n_samples);
    const int band = c.mode == MODE_GREY ? 0 : sid / c.nq;
    const float2 *sp = c.sur + fs * nw;
    for (int i = t; i < nw; i += kTableThreads) s_sur[i] = sp[i];
    for (int i = t; i <= nw; i += kTableThreads) s_fw[i] = c.fw[i];
    // sweep thread: hemisphere h (0: towards the west wall), node m
    const int h = t >= kSurNodes ? 1 : 0, m = t - h * kSurNodes;
    float invmu = 0.0f, F = 0.0f;
    if (t < 2 * kSurNodes) {
        const float u = (float)m * (1.0f / (float)kSurBins);
        const float mu = m ? u * u : 9.31322574615478516e-10f;  // 2^-30
        invmu = 1.0f / mu;
        F = c.mode == MODE_GREY ? c.Tw4[h] : __ldg(c.ibw + h * c.nbands + band);
    }
    __syncthreads();
    for (int step = 0; step < nw; ++step) {
        if (t < 2 * kSurNodes) {
            const int l = h ? nw - 1 - step : step;
            const float2 kv = s_sur[l];
            const float f0 = s_fw[l], f1 = s_fw[l + 1];
            const float o = (f0 + f1) * 0.5f;
            const float half = h ? (f1 - o) * invmu : (o - f0) * invmu;
            const float e1h = mc_expm1(-(kv.x * half));
            s_val[h][m] = make_float2(fmaf(e1h, F - kv.y, F), -e1h);
            const float e1 = mc_expm1(-(kv.x * ((f1 - f0) * invmu)));
            F = fmaf(e1, F - kv.y, F);
        }
        __syncthreads();
        if (t < 2 * kSurBins) {
            const int hb = t / kSurBins, mb = t - hb * kSurBins;
            const int l = hb ? nw - 1 - step : step;
            const float2 v0 = s_val[hb][mb], v1 = s_val[hb][mb + 1];
            const float dJ = v1.x - v0.x, dA = v1.y - v0.y;
            c.surtab[(fs * nw + l) * (2 * kSurBins) + t] = make_float4(v0.x, dJ, v0.y, dA);
            const float w0 = (float)(3 * (2 * mb + 1)), w1 = (float)(3 * mb + 2);
            float2 eJ = ff_add(ff_mul(w0, v0.x), ff_mul(w1, dJ));
            float2 eA = ff_add(ff_mul(w0, v0.y), ff_mul(w1, dA));
            for (int o = 16; o > 0; o >>= 1) {
                float2 pJ, pA;
                pJ.x = __shfl_xor_sync(0xffffffffu, eJ.x, o);
                pJ.y = __shfl_xor_sync(0xffffffffu, eJ.y, o);
                pA.x = __shfl_xor_sync(0xffffffffu, eA.x, o);
                pA.y = __shfl_xor_sync(0xffffffffu, eA.y, o);
                eJ = ff_add(eJ, pJ);
                eA = ff_add(eA, pA);
            }
            if ((t & 31) == 0)
                s_half[t >> 5] = make_double2((double)eJ.x + (double)eJ.y, (double)eA.x + (double)eA.y);
        }
        __syncthreads();
        if (t < 2) {  // the step's two layers
            const int l = t ? nw - 1 - step : step;
            s_mean[2 * l + t] = make_double2(s_half[2 * t].x + s_half[2 * t + 1].x,
                                             s_half[2 * t].y + s_half[2 * t + 1].y);
        }
    }
    __syncthreads();
    // both hemispheres, weight 1/2; the sums carry the factor 3
    const double sc = 0.5 / (3.0 * (double)kSurBins * (double)kSurBins);
    for (int l = t; l < nw; l += kTableThreads) {
        const double2 a = s_mean[2 * l], b = s_mean[2 * l + 1];
        const double J = (a.x + b.x) * sc, A = (a.y + b.y) * sc;
        const float Jhi = (float)J;
        const long long idx = fs * nw + l;
        c.Jhat[idx] = make_double2(J, A);
        c.Jf[idx] = make_float4(Jhi, (float)(J - (double)Jhi), (float)A, s_sur[l].y);
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
// table coordinates (weights wt_a in T, wx_b in x; sum_a' wt_a' = 1),
//   E[Y_a] = sum_s C_s k_s (Ib_s - Jhat_s(w))
//          = sum_{b,a,a'} wx_b wt_a wt_a' Da(w)[t][x_b][a][a'],
//   E[Y_b] = sum_s C_s Ahat_s(w) k_s (Ib_s - Ibar_s(w))
//          = sum_{b,a,a'} wx_b wt_a wt_a' Db(w)[t][x_b][a][a'],
// with the node sums per (field, group, layer) and table cell (t, x)
//   Da[t][x][a][a'] = sum_s C_s k_s[t+a][x] (Ib_s[t+a'] - Jhat_s),
//   Db[t][x][a][a'] = sum_s C_s Ahat_s k_s[t+a][x] (Ib_s[t+a'] - Ibar_s):
// a cell needs 16 node sums per group instead of a pass over the group's
// samples, and the differences Ib - Jhat, where optically thick samples
// cancel, are formed per sample before any sum.  Arithmetic in float pairs
// (hi + lo, about 48 bits: error-free products by fma and error-free sums;
// this file is compiled without FMA contraction), at FP32 rates -- this
// GPU's FP64 rate is a small fraction of them.  The cell's weights are
// formed in FP64 and its 16-term combination summed in pairs.
// ---------------------------------------------------------------------------
struct NodeLayout {
    int nTc, per;  // table cells (t, x), pairs per (field, group, layer): Da then Db, 4 each per cell
};
__host__ __device__ inline NodeLayout node_layout(const CvParams &c) {
    NodeLayout L;
    L.nTc = (c.nT - 1) * c.nX;
    L.per = L.nTc * 8;
    return L;
}

long long cv_node_count(const CvParams &c) {
    const NodeLayout L = node_layout(c);
    const long long niR = c.ew1 - c.ew0;
    return (long long)c.nfields * c.n_groups * niR * L.per;
}

// a double as a float pair
__device__ __forceinline__ float2 ff_of(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}
// a pair times a float (the low part's product rounded)
__device__ __forceinline__ float2 ff_mulf(float2 a, float b) {
    const float p = a.x * b;
    return make_float2(p, fmaf(a.x, b, -p) + a.y * b);
}
// a pair times a pair
__device__ __forceinline__ float2 ff_mulff(float2 a, float2 b) {
    const float p = a.x * b.x;
    return make_float2(p, fmaf(a.x, b.x, -p) + (a.x * b.y + a.y * b.x));
}
// a float minus a pair, as a pair
__device__ __forceinline__ float2 ff_fsub(float a, float2 b) { return ff_add(make_float2(a, 0.0f), make_float2(-b.x, -b.y)); }

// Blocks: (field, group, region layer).  Work units: the table cells (t, x),
// each with its eight sums, one per thread in rounds of blockDim.  The
// per-sample weights and the inputs of the differences come from shared
// memory in chunks of 256 samples.
__global__ void __launch_bounds__(256) cv_nodes_kernel(const CvParams c) {
    __shared__ int s_ib[256];      // band * nT
    __shared__ int s_koff[256];    // sample * nT * nX
    __shared__ float2 s_C[256], s_CA[256], s_J[256];  // C, C Ahat, Jhat as pairs
    __shared__ float s_Ibar[256];
    const NodeLayout L = node_layout(c);
    const int niR = c.ew1 - c.ew0;
    const long long b = blockIdx.x;
    const int wR = (int)(b % niR);
    const long long fg = b / niR;
    const int g = (int)(fg % c.n_groups);
    const int f = (int)(fg / c.n_groups);
    const int w = c.ew0 + wR;
    float2 *out = reinterpret_cast<float2 *>(c.nodes) + b * L.per;
    const int q0 = c.grp_start[g], q1 = c.grp_start[g + 1];
    for (int u0 = 0; u0 < L.nTc; u0 += blockDim.x) {
        const int u = u0 + threadIdx.x;
        const int t = u / c.nX, x = u - t * c.nX;
        float2 acc[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) acc[r] = make_float2(0.0f, 0.0f);
        for (int qc = q0; qc < q1; qc += 256) {
            const int nq = min(256, q1 - qc);
            __syncthreads();
            if ((int)threadIdx.x < nq) {
                const int q = qc + threadIdx.x;
                const int sid = c.samp_id[q];
                const double C = c.samp_C[q];
                const long long o = ((long long)f * c.n_samples + sid) * c.nw + w;
                const double2 jh = c.Jhat[o];
                s_ib[threadIdx.x] = (sid / c.nq) * c.nT;
                s_koff[threadIdx.x] = sid * c.nT * c.nX;
                s_C[threadIdx.x] = ff_of(C);
                s_CA[threadIdx.x] = ff_of(C * jh.y);
                s_J[threadIdx.x] = ff_of(jh.x);
                s_Ibar[threadIdx.x] = c.sur[o].y;
            }
            __syncthreads();
            if (u >= L.nTc) continue;
            for (int j = 0; j < nq; ++j) {
                const float *kk = c.ktab + s_koff[j] + t * c.nX + x;
                const float *ib = c.ibtab + s_ib[j] + t;
                const float k0 = __ldg(kk), k1 = __ldg(kk + c.nX);
                const float i0 = __ldg(ib), i1 = __ldg(ib + 1);
                const float2 J = s_J[j];
                const float Ibar = s_Ibar[j];
                const float2 da0 = ff_fsub(i0, J), da1 = ff_fsub(i1, J);
                const float2 db0 = ff_fsub(i0, make_float2(Ibar, 0.0f)), db1 = ff_fsub(i1, make_float2(Ibar, 0.0f));
                const float2 ck0 = ff_mulf(s_C[j], k0), ck1 = ff_mulf(s_C[j], k1);
                const float2 ca0 = ff_mulf(s_CA[j], k0), ca1 = ff_mulf(s_CA[j], k1);
                acc[0] = ff_add(acc[0], ff_mulff(ck0, da0));
                acc[1] = ff_add(acc[1], ff_mulff(ck0, da1));
                acc[2] = ff_add(acc[2], ff_mulff(ck1, da0));
                acc[3] = ff_add(acc[3], ff_mulff(ck1, da1));
                acc[4] = ff_add(acc[4], ff_mulff(ca0, db0));
                acc[5] = ff_add(acc[5], ff_mulff(ca0, db1));
                acc[6] = ff_add(acc[6], ff_mulff(ca1, db0));
                acc[7] = ff_add(acc[7], ff_mulff(ca1, db1));
            }
        }
        if (u < L.nTc) {  // layout: Da [t][x][a*2 + a'], then Db alike
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                out[(long long)u * 4 + r] = acc[r];
                out[(long long)L.nTc * 4 + (long long)u * 4 + r] = acc[4 + r];
            }
        }
    }
}

// E[Y] per (field, cell) from the node sums, all groups.
__global__ void cv_mean_nodes_kernel(const CvParams c) {
    const NodeLayout L = node_layout(c);
    const int njR = c.ea1 - c.ea0, nkR = c.eb1 - c.eb0, niR = c.ew1 - c.ew0;
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
        // the cell's interpolation weights w4[bx][a][a'] = wx[bx] wt[a] wt[a']
        // (the product of the k and Ib interpolations), formed once for all
        // groups
        float2 w4[2][4];
        for (int bx = 0; bx < nb; ++bx)
            for (int a = 0; a < 2; ++a)
                for (int a2 = 0; a2 < 2; ++a2) w4[bx][a * 2 + a2] = ff_of(wx[bx] * wt[a] * wt[a2]);
        for (int g = 0; g < c.n_groups; ++g) {
            const float2 *lay = reinterpret_cast<const float2 *>(c.nodes) +
                                (((long long)f * c.n_groups + g) * niR + iR) * L.per;
            float2 ea = make_float2(0.0f, 0.0f), eb = make_float2(0.0f, 0.0f);
            for (int bx = 0; bx < nb; ++bx) {
                const long long o = ((long long)ti * c.nX + xi + bx) * 4;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    ea = ff_add(ea, ff_mulff(w4[bx][q], __ldg(lay + o + q)));
                    eb = ff_add(eb, ff_mulff(w4[bx][q], __ldg(lay + (long long)L.nTc * 4 + o + q)));
                }
            }
            c.muY[((long long)f * c.n_groups + g) * c.region_cells + tc] =
                make_double2((double)ea.x + (double)ea.y, (double)eb.x + (double)eb.y);
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
    // one block per (field, sample); its shared memory beyond 48 KB was
    // allowed once per device (cv_table_allow_smem), outside any capture
    const size_t smem = cv_table_smem(c.nw);
    cv_table_kernel<<<(unsigned)((long long)c.nfields * c.n_samples), kTableThreads, smem, st>>>(c);
    return (int)cudaGetLastError();
}

// The table kernel's dynamic shared memory for the largest grid the control
// variate takes (imax 4096), set once per device.
int cv_table_allow_smem() {
    return (int)cudaFuncSetAttribute(cv_table_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)cv_table_smem(kCvMaxPlanes));
}

int launch_cv_mean(const CvParams &c, void *stream) {
    const long long n = (long long)c.nfields * c.region_cells;
    cudaStream_t st = (cudaStream_t)stream;
    if (c.nodes) {  // tables without particles: node sums, then the cells
        const long long blocks = (long long)c.nfields * c.n_groups * (c.ew1 - c.ew0);
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
    const unsigned tiles = (unsigned)(((q.njR + kFinTile - 1) / kFinTile) * ((q.niR + kFinTile - 1) / kFinTile));
    if (tiles == 0 || q.nkR <= 0 || q.nfields <= 0) return (int)cudaGetLastError();
    dnsmc::note_launch();
    finalize_kernel<<<dim3(tiles, (unsigned)q.nkR, (unsigned)q.nfields), kFinTile * kFinRows, 0, st>>>(q);
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
