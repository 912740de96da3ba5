// mc_cvnet.cu -- the learned part of the control variate.
//
// A small MLP maps, per cell and band group, local features of the medium to
// the quantities the Monte Carlo estimator needs but cannot know in advance:
//
//   out[4g+0], out[4g+1] (g < 16 band-group slots): offsets of the control-variate coefficients from
//       (beta_a, beta_b) = (1, -1); any finite pair keeps the estimate
//       unbiased (E[Y_a], E[Y_b] are exact), the best pair minimises the
//       variance of X - beta_a Y_a - beta_b Y_b;
//   out[4g+2]: log of the estimator variance per ray of the cell (scale S_v);
//   out[4g+3]: log of the ray-voxel steps per ray of its packet (scale S_c);
//
// the last two drive the ray allocation n ~ sqrt(v / c) per (band group,
// packet) at a fixed expected step budget.  The network never enters the
// estimate itself: a poor network costs variance, not bias.
//
// Features (67, padded with zeros to 80): T and x_H2O of the cell, its signed
// wall-normal position 2 eta - 1, and T and x_H2O at 32 points of the
// wall-normal line through the cell (layers ((2q+1) nw) / 64), all mapped to
// [-1, 1] by the table's T and x ranges.  Layers 67 -> 128 -> 128 -> 128 -> 64
// with GELU (tanh form), BF16 weights and activations, FP32 accumulation on
// the fifth-generation tensor cores (tcgen05.mma, accumulators in tensor
// memory; mc_cvnet_tc.cuh): the forward pass (inference with the features
// and the coefficient epilogue fused in; training with its saves) and the
// backward GEMMs.  Training: a loss kernel writes dL/dout; the backward pass
// runs dW = dZ^T H (split over the batch with a deterministic reduction) and
// dH = dZ W with the GELU derivative fused, and Adam updates FP32 master
// weights.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/dnsmc.h"
#include "mc_internal.h"

namespace dnsmc {
int report_error(int code, const char *msg);
}

using namespace dnsmc;

namespace {

typedef __nv_bfloat16 bf16;

constexpr int NFEAT = 67;
constexpr int K0 = 80;       // padded input width (multiple of 16)
constexpr int HID = 128;
constexpr int NOUT = 64;     // 16 group slots x 4 heads
constexpr int MAXG = 16;
constexpr int NPROF = 32;
constexpr int NLAB = 8;      // labels per (cell, group): Cxx Caa Cbb Cxa Cxb Cab v c

// flat parameter layout (FP32 master), weights row-major [out][in]
constexpr long long OFF_W1 = 0;
constexpr long long OFF_B1 = OFF_W1 + (long long)HID * K0;
constexpr long long OFF_W2 = OFF_B1 + HID;
constexpr long long OFF_B2 = OFF_W2 + (long long)HID * HID;
constexpr long long OFF_W3 = OFF_B2 + HID;
constexpr long long OFF_B3 = OFF_W3 + (long long)HID * HID;
constexpr long long OFF_W4 = OFF_B3 + HID;
constexpr long long OFF_B4 = OFF_W4 + (long long)NOUT * HID;
constexpr long long NPARAM = OFF_B4 + NOUT;

// bf16 weight copy layout (weights only, same order)
constexpr long long WOFF_1 = 0;
constexpr long long WOFF_2 = WOFF_1 + (long long)HID * K0;
constexpr long long WOFF_3 = WOFF_2 + (long long)HID * HID;
constexpr long long WOFF_4 = WOFF_3 + (long long)HID * HID;
constexpr long long NWEIGHT = WOFF_4 + (long long)NOUT * HID;


#define CK(x)                                                                        \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess) return cuda_fail(#x, e_);                             \
    } while (0)
#define RTRY(x)                      \
    do {                             \
        int rc_ = (x);               \
        if (rc_ != DNSMC_OK) return rc_; \
    } while (0)

int cuda_fail(const char *what, cudaError_t e) {
    char msg[256];
    snprintf(msg, sizeof msg, "%s failed: %s", what, cudaGetErrorString(e));
    return report_error(DNSMC_ERR_CUDA, msg);
}
int arg_fail(const char *msg) { return report_error(DNSMC_ERR_ARG, msg); }
int state_fail(const char *msg) { return report_error(DNSMC_ERR_STATE, msg); }

// GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units",
// 2016): 0.5 z (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3), within
// 5e-4 of the erf form (below the bf16 rounding of the activations),
// written as z - z / (1 + e^(2u)) with the hardware exponential.
__device__ __forceinline__ float gelu_u(float z) { return 0.7978845608028654f * fmaf(0.044715f * z, z * z, z); }
__device__ __forceinline__ float gelu(float z) { return z - __fdividef(z, __expf(2.0f * gelu_u(z)) + 1.0f); }
// its derivative: s + z s (1 - s) 2 u'(z), s = 1 / (1 + e^(-2u)) the sigmoid
// of 2u, u' = sqrt(2/pi) (1 + 3 * 0.044715 z^2)
__device__ __forceinline__ float gelu_grad(float z) {
    const float sg = __fdividef(1.0f, 1.0f + __expf(-2.0f * gelu_u(z)));
    const float du = 0.7978845608028654f * fmaf(0.134145f * z, z, 1.0f);
    return fmaf(z * sg * (1.0f - sg), 2.0f * du, sg);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// ---------------------------------------------------------------------------
// Features
// ---------------------------------------------------------------------------
struct FeatParams {
    int nw, na, nb, mode;
    const float *fT;
    const float2 *fTX;
    const float *fw;
    long long field_stride;
    int ew0, ea0, eb0, niR, njR, nkR;
    long long region_cells;
    int nfields;
    float Tc, Tis, Xc, Xis;   // x' = (x - c) * is
    bf16 *out;                // [f * region_cells + tc][K0]
};

// The K0 bf16 features of row r (field f, cell tc of the region in tally
// order), packed pairwise: the features kernel and the tensor-memory
// forward both use this, so their features are the same bits.
__device__ __forceinline__ void feature_row(const FeatParams &P, long long r, uint32_t (&out)[K0 / 2]) {
    const int f = (int)(r / P.region_cells);
    const long long tc = r - (long long)f * P.region_cells;
    const int jR = (int)(tc % P.njR);
    const long long t = tc / P.njR;
    const int kR = (int)(t % P.nkR);
    const int iR = (int)(t / P.nkR);
    const int i = P.ew0 + iR, j = P.ea0 + jR, k = P.eb0 + kR;
    const long long base = (long long)f * P.field_stride + (long long)k * P.na + j;
    const long long plane = (long long)P.na * P.nb;
    float feat[K0];
#pragma unroll
    for (int q = 0; q < K0; ++q) feat[q] = 0.0f;
    float T, X = 0.0f;
    if (P.mode == MODE_TX) {
        const float2 v = P.fTX[base + i * plane];
        T = v.x; X = v.y;
    } else {
        T = P.fT[base + i * plane];
    }
    feat[0] = __fmul_rn(__fsub_rn(T, P.Tc), P.Tis);
    feat[1] = P.mode == MODE_TX ? __fmul_rn(__fsub_rn(X, P.Xc), P.Xis) : 0.0f;
    const float o = __fmul_rn(0.5f, __fadd_rn(P.fw[i], P.fw[i + 1]));
    const float eta = __fdiv_rn(__fsub_rn(o, P.fw[0]), __fsub_rn(P.fw[P.nw], P.fw[0]));
    feat[2] = __fsub_rn(__fmul_rn(2.0f, eta), 1.0f);
#pragma unroll
    for (int q = 0; q < NPROF; ++q) {
        const int l = ((2 * q + 1) * P.nw) / (2 * NPROF);
        if (P.mode == MODE_TX) {
            const float2 v = P.fTX[base + l * plane];
            feat[3 + q] = __fmul_rn(__fsub_rn(v.x, P.Tc), P.Tis);
            feat[3 + NPROF + q] = __fmul_rn(__fsub_rn(v.y, P.Xc), P.Xis);
        } else {
            feat[3 + q] = __fmul_rn(__fsub_rn(P.fT[base + l * plane], P.Tc), P.Tis);
        }
    }
#pragma unroll
    for (int q = 0; q < K0 / 2; ++q) out[q] = pack_bf16(feat[2 * q], feat[2 * q + 1]);
}

__global__ void features_kernel(const FeatParams P) {
    const long long n = (long long)P.nfields * P.region_cells;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
         r += (long long)gridDim.x * blockDim.x) {
        uint32_t packed[K0 / 2];
        feature_row(P, r, packed);
        uint32_t *dst = reinterpret_cast<uint32_t *>(P.out + r * K0);
#pragma unroll
        for (int q = 0; q < K0 / 2; ++q) dst[q] = packed[q];
    }
}

struct GemmParams {
    int M, N, K, klen;        // klen: K range per split
    const bf16 *A;
    long long a_sm, a_sk;
    const bf16 *B;
    long long b_sk, b_sn;
    float *C;                 // partials [split][M][N]
    const float *Z;           // [M][N] pre-activation for the fused GELU' epilogue
    bf16 *D;                  // [M][N]
};

// grad[off + e] = sum over splits of partials (fixed order)
__global__ void reduce_splits_kernel(const float *part, int splits, long long n, float *grad) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int z = 0; z < splits; ++z) s += part[z * n + e];
        grad[e] = s;
    }
}

// db[n] = sum over rows of dZ[row][n]; one block per column, fixed tree order
__global__ void colsum_kernel(const bf16 *dZ, long long rows, int ncol, float *db) {
    __shared__ float red[256];
    const int n = blockIdx.x;
    float s = 0.0f;
    for (long long r = threadIdx.x; r < rows; r += blockDim.x) s += __bfloat162float(dZ[r * ncol + n]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[n] = red[0];
}

// ---------------------------------------------------------------------------
// Loss: per row and band-group slot g < G
//   beta loss  (V(beta) + ridge (Caa da^2 + Cbb db^2)) / S_beta
//   var loss   (v / S_v) exp(-o_v) + o_v     (minimiser: o_v = log E[v / S_v])
//   cost loss  (c / S_c) exp(-o_c) + o_c
// mean over rows; dOut = d(mean)/d out, written as bf16.
// ---------------------------------------------------------------------------
struct LossParams {
    long long rows, nvalid;
    int G;
    const float *out;         // [rows][NOUT]
    const float *lab;         // [*][G][NLAB]
    const int *idx;           // row r -> label row idx[r]
    float Sbeta, Sv, Sc, ridge;
    bf16 *dout;               // [rows][NOUT]
    double *part;             // per block: beta, var, cost loss sums
};

__device__ __forceinline__ float clampo(float o) { return fminf(fmaxf(o, -15.0f), 15.0f); }

__global__ void loss_kernel(const LossParams L) {
    __shared__ double red[3][256];
    double lb = 0.0, lv = 0.0, lc = 0.0;
    const float inv = 1.0f / (float)max(1LL, L.nvalid);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < L.rows;
         r += (long long)gridDim.x * blockDim.x) {
        float d[NOUT];
#pragma unroll
        for (int q = 0; q < NOUT; ++q) d[q] = 0.0f;
        if (r < L.nvalid) {
            const long long lr = L.idx ? (long long)L.idx[r] : r;
            for (int g = 0; g < L.G; ++g) {
                const float *y = L.lab + (lr * L.G + g) * NLAB;
                const float *o = L.out + r * NOUT + 4 * g;
                const float Cxx = y[0], Caa = y[1], Cbb = y[2], Cxa = y[3], Cxb = y[4], Cab = y[5];
                const float da = o[0], db = o[1];
                const float ba = 1.0f + da, bb = -1.0f + db;
                const float V = Cxx - 2.0f * ba * Cxa - 2.0f * bb * Cxb + ba * ba * Caa + 2.0f * ba * bb * Cab +
                                bb * bb * Cbb;
                lb += (double)((V + L.ridge * (Caa * da * da + Cbb * db * db)) / L.Sbeta);
                d[4 * g + 0] = (2.0f * (ba * Caa + bb * Cab - Cxa) + 2.0f * L.ridge * Caa * da) / L.Sbeta * inv;
                d[4 * g + 1] = (2.0f * (bb * Cbb + ba * Cab - Cxb) + 2.0f * L.ridge * Cbb * db) / L.Sbeta * inv;
                if (y[6] > 0.0f) {
                    const float ov = clampo(o[2]), e = y[6] / L.Sv * expf(-ov);
                    lv += (double)(e + ov);
                    d[4 * g + 2] = (1.0f - e) * inv;
                }
                if (y[7] > 0.0f) {
                    const float oc = clampo(o[3]), e = y[7] / L.Sc * expf(-oc);
                    lc += (double)(e + oc);
                    d[4 * g + 3] = (1.0f - e) * inv;
                }
            }
        }
        uint32_t *dst = reinterpret_cast<uint32_t *>(L.dout + r * NOUT);
#pragma unroll
        for (int q = 0; q < NOUT / 2; ++q) dst[q] = pack_bf16(d[2 * q], d[2 * q + 1]);
    }
    red[0][threadIdx.x] = lb; red[1][threadIdx.x] = lv; red[2][threadIdx.x] = lc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) L.part[blockIdx.x * 3 + q] = red[q][0];
}

// Adam on the FP32 master copy; bf16 copy of the weights.
__global__ void adam_kernel(float *p, const float *grad, float *m, float *v, bf16 *w, long long n, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float gr = grad[e];
        const float mm = b1 * m[e] + (1.0f - b1) * gr;
        const float vv = b2 * v[e] + (1.0f - b2) * gr * gr;
        m[e] = mm;
        v[e] = vv;
        const float upd = lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        p[e] -= upd;
    }
}

// bf16 copies of the weight blocks of the master array: w[0, NWEIGHT) row
// major per matrix ([out][in], the warp-level kernels), w[NWEIGHT, 2 NWEIGHT)
// in the tensor-core order [in/8][out][8] of the tcgen05 forward (the same
// block offsets)
__host__ __device__ __forceinline__ long long tc_order(long long e) {
    long long off, rows, cols;
    if (e < WOFF_2) { off = WOFF_1; rows = HID; cols = K0; }
    else if (e < WOFF_3) { off = WOFF_2; rows = HID; cols = HID; }
    else if (e < WOFF_4) { off = WOFF_3; rows = HID; cols = HID; }
    else { off = WOFF_4; rows = NOUT; cols = HID; }
    const long long q = e - off, n = q / cols, k = q % cols;
    return off + (k >> 3) * rows * 8 + n * 8 + (k & 7);
}

__global__ void weights_to_bf16_kernel(const float *p, bf16 *w) {
    const long long n = NWEIGHT;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        long long src;
        if (e < WOFF_2) src = OFF_W1 + e;
        else if (e < WOFF_3) src = OFF_W2 + (e - WOFF_2);
        else if (e < WOFF_4) src = OFF_W3 + (e - WOFF_3);
        else src = OFF_W4 + (e - WOFF_4);
        const bf16 v = __float2bfloat16(p[src]);
        w[e] = v;
        w[NWEIGHT + tc_order(e)] = v;
    }
}

// ---------------------------------------------------------------------------
// Training labels from a solve with per-ray moments: per (row = region cell in
// tally order, g) the centred per-ray covariances of (X, Y_a, Y_b), the
// estimator variance per ray (var of the group mean x rays) and the steps
// per ray of the cell's packet.
// ---------------------------------------------------------------------------
struct LabelParams {
    int nfields, G, niR, njR, nkR, tile_a, tile_b, npa, npb, n_packets;
    long long region_cells;
    const double *moments;    // [f][g][tc][9]
    const double *varg;       // [f][g][dense cell]
    const unsigned long long *steps;  // [f][g][p]
    int rays;
    const int *rays_item;
    int rays_gstride;
    float *lab;               // [f * region_cells + tc][G][NLAB]
};

__global__ void labels_kernel(const LabelParams L) {
    const long long n = (long long)L.nfields * L.region_cells;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
         r += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(r / L.region_cells);
        const long long tc = r - (long long)f * L.region_cells;
        const int jR = (int)(tc % L.njR);
        const long long t = tc / L.njR;
        const int kR = (int)(t % L.nkR);
        const int iR = (int)(t / L.nkR);
        const int p = (iR * L.npb + kR / L.tile_b) * L.npa + jR / L.tile_a;
        const long long dense = iR + (long long)L.niR * (jR + (long long)L.njR * kR);
        for (int g = 0; g < L.G; ++g) {
            const int N = L.rays_item ? L.rays_item[g * L.rays_gstride + p] : L.rays;
            float *y = L.lab + (r * L.G + g) * NLAB;
            if (N < 2) {
                for (int q = 0; q < NLAB; ++q) y[q] = 0.0f;
                continue;
            }
            const double *mo = L.moments + (((long long)f * L.G + g) * L.region_cells + tc) * 9;
            const double in = 1.0 / N;
            const double mx = mo[0] * in, ma = mo[1] * in, mb = mo[2] * in;
            y[0] = (float)fmax(0.0, mo[3] * in - mx * mx);
            y[1] = (float)fmax(0.0, mo[4] * in - ma * ma);
            y[2] = (float)fmax(0.0, mo[5] * in - mb * mb);
            y[3] = (float)(mo[6] * in - mx * ma);
            y[4] = (float)(mo[7] * in - mx * mb);
            y[5] = (float)(mo[8] * in - ma * mb);
            y[6] = (float)(L.varg[((long long)f * L.G + g) * L.region_cells + dense] * N);
            y[7] = (float)((double)L.steps[((long long)f * L.G + g) * L.n_packets + p] * in);
        }
    }
}

// ---------------------------------------------------------------------------
// Inference: network outputs -> coefficient pairs (tally layout) and per-cell
// (v, c); per (group, packet) allocation weights; ray counts.
// ---------------------------------------------------------------------------
// The coefficient epilogue of dnsmc_cvnet_apply (fused into the tcgen05
// forward): per row and band group, beta = (1, -1) + the first two outputs
// (non-finite: (1, -1)) and (v, c) = (S_v e^o2, S_c e^o3), o clamped to 15.
struct ApplyParams {
    long long rows;           // nfields * region_cells
    int G;
    const float *out;
    float Sv, Sc;
    float2 *beta;             // [f][g][tc] or null
    float2 *vc;               // [f][g][tc] (v, c)
    long long region_cells;
};

}  // namespace
#include "mc_cvnet_tc.cuh"
namespace {

struct AllocParams {
    int nfields, G, n_packets, npa, npb, tile_a, tile_b, njR, nkR;
    long long region_cells;
    const float2 *vc;
    float *wgt;               // [g][p]: sqrt(v_sum / c)
    float *cost;              // [g][p]: c (steps per packet-ray)
};

// one warp per (g, p): v summed over the packet's cells and fields, c averaged
__global__ void alloc_weights_kernel(const AllocParams A) {
    const int lane = threadIdx.x & 31;
    const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long it = wid; it < (long long)A.G * A.n_packets; it += nw) {
        const int g = (int)(it / A.n_packets), p = (int)(it % A.n_packets);
        const int pa = p % A.npa, rest = p / A.npa, pb = rest % A.npb, pw = rest / A.npb;
        float vs = 0.0f, cs = 0.0f, na = 0.0f;
        for (int cl = lane; cl < A.tile_a * A.tile_b; cl += 32) {  // the packet's cells
            const int jR = pa * A.tile_a + cl % A.tile_a, kR = pb * A.tile_b + cl / A.tile_a;
            if (jR >= A.njR || kR >= A.nkR) continue;
            const long long tc = ((long long)pw * A.nkR + kR) * A.njR + jR;
            for (int f = 0; f < A.nfields; ++f) {
                const float2 x = A.vc[((long long)f * A.G + g) * A.region_cells + tc];
                vs += x.x;
                cs += x.y;
                na += 1.0f;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            vs += __shfl_xor_sync(0xffffffffu, vs, o);
            cs += __shfl_xor_sync(0xffffffffu, cs, o);
            na += __shfl_xor_sync(0xffffffffu, na, o);
        }
        if (lane == 0) {
            const float c = na > 0.0f ? cs / na : 1.0f;
            A.wgt[it] = sqrtf(vs / fmaxf(c, 1e-3f));
            A.cost[it] = c;
        }
    }
}

// lambda = mean_rays * sum(c) / sum(w c), in FP64 and in a fixed order: each
// of kScaleBlocks blocks sums its grid-strided share and writes its partial
// sums; the last block to finish adds the partials in block order (the
// result does not depend on which block that is) and re-arms the counter.
constexpr int kScaleBlocks = 152, kScaleThreads = 256;
__global__ void __launch_bounds__(kScaleThreads) alloc_scale_kernel(const float *wgt, const float *cost, long long n,
                                                                   float mean_rays, float *lam, double2 *part,
                                                                   unsigned int *done) {
    __shared__ double r0[kScaleThreads], r1[kScaleThreads];
    __shared__ bool last;
    double a = 0.0, b = 0.0;
    for (long long e = blockIdx.x * (long long)kScaleThreads + threadIdx.x; e < n;
         e += (long long)kScaleBlocks * kScaleThreads) {
        a += (double)cost[e];
        b += (double)wgt[e] * cost[e];
    }
    r0[threadIdx.x] = a; r1[threadIdx.x] = b;
    __syncthreads();
    for (int w = kScaleThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) { r0[threadIdx.x] += r0[threadIdx.x + w]; r1[threadIdx.x] += r1[threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = make_double2(r0[0], r1[0]);
        __threadfence();
        last = atomicAdd(done, 1u) == (unsigned)(kScaleBlocks - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    a = 0.0; b = 0.0;
    for (int i = threadIdx.x; i < kScaleBlocks; i += kScaleThreads) {
        const double2 v = __ldcg(part + i);
        a += v.x;
        b += v.y;
    }
    r0[threadIdx.x] = a; r1[threadIdx.x] = b;
    __syncthreads();
    for (int w = kScaleThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) { r0[threadIdx.x] += r0[threadIdx.x + w]; r1[threadIdx.x] += r1[threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *lam = r1[0] > 0.0 ? (float)(mean_rays * r0[0] / r1[0]) : 0.0f;
        *done = 0u;
    }
}

__global__ void alloc_rays_kernel(const float *wgt, long long n, const float *lam, int B, int nmin, int nmax,
                                  int *rays) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float x = *lam * wgt[e];
        int r = (int)rintf(x / (float)B) * B;
        if (!(x == x)) r = nmin;
        r = min(max(r, nmin), nmax);
        rays[e] = r;
    }
}

inline int grid1(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    return (int)std::max(1LL, std::min(b, 152LL * 32));
}

}  // namespace

// ===========================================================================
// Host side
// ===========================================================================
template <class T>
struct NBuf {
    T *p = nullptr;
    size_t n = 0;
    int ensure(size_t m) {
        if (m <= n) return DNSMC_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(m, 1) * sizeof(T));
        if (e != cudaSuccess) return cuda_fail("cudaMalloc", e);
        n = m;
        return DNSMC_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct dnsmc_cvnet {
    dnsmc_cvnet_config cfg;
    int device = 0;
    cudaStream_t stream = nullptr;
    NBuf<float> P, grad, m, v;
    NBuf<bf16> W;
    long long step = 0;
    float Sbeta = 0.f, Sv = 0.f, Sc = 0.f;      // label scales (set from the first data)
    // dataset
    long long nrows = 0;
    NBuf<bf16> dX;
    NBuf<float> dlab;
    int dG = 0;
    // work buffers
    long long cap_rows = 0;
    NBuf<int> idx;
    NBuf<bf16> H0, H1, H2, H3, dO, dZ3, dZ2, dZ1;
    NBuf<float> Z1, Z2, Z3, out, part;
    NBuf<double> lpart;
    // inference
    NBuf<bf16> iX;
    NBuf<float> iout;
    NBuf<float2> vc;
    NBuf<float> wgt, cost, lam;
    NBuf<double2> lam_part;          // alloc_scale_kernel: per-block partial sums
    NBuf<unsigned int> lam_done;     // and its finished-block counter
    NBuf<unsigned int> status;                // DNSMC_STATUS_* bits of the tensor-memory forward
    std::mt19937_64 rng;
    ~dnsmc_cvnet() {
        P.release(); grad.release(); m.release(); v.release(); W.release(); dX.release(); dlab.release();
        idx.release(); H0.release(); H1.release(); H2.release(); H3.release(); dO.release(); dZ3.release();
        dZ2.release(); dZ1.release(); Z1.release(); Z2.release(); Z3.release(); out.release(); part.release();
        lpart.release(); iX.release(); iout.release(); vc.release(); wgt.release(); cost.release(); lam.release();
        lam_part.release(); lam_done.release();
        status.release();
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int set_dev(dnsmc_cvnet *n) {
    CK(cudaSetDevice(n->device));
    return DNSMC_OK;
}

// The tcgen05 forward (mc_cvnet_tc.cuh): one CTA per SM, persistent.
int launch_forward_tc(TcParams &F, dnsmc_cvnet *n, cudaStream_t st) {
    static int attr = 0;
    if (!attr) {
        CK(cudaFuncSetAttribute(mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
        attr = 1;
    }
    const long long tiles = (F.rows + TC_TILE - 1) / TC_TILE;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = (int)std::max(1LL, std::min((long long)sms, (tiles + TC_WG - 1) / TC_WG));
    F.Wtc = n->W.p + NWEIGHT;
    F.P = n->P.p;
    F.status = n->status.p;
    dnsmc::note_launch();
    mlp_tc_kernel<<<blocks, TC_THREADS, TC_SMEM, st>>>(F);
    CK(cudaGetLastError());
    return DNSMC_OK;
}

int ensure_work(dnsmc_cvnet *n, long long rows) {
    if (rows <= n->cap_rows) return DNSMC_OK;
    RTRY(n->idx.ensure(rows)); RTRY(n->H0.ensure(rows * K0));
    RTRY(n->H1.ensure(rows * HID)); RTRY(n->H2.ensure(rows * HID)); RTRY(n->H3.ensure(rows * HID));
    RTRY(n->Z1.ensure(rows * HID)); RTRY(n->Z2.ensure(rows * HID)); RTRY(n->Z3.ensure(rows * HID));
    RTRY(n->dZ1.ensure(rows * HID)); RTRY(n->dZ2.ensure(rows * HID)); RTRY(n->dZ3.ensure(rows * HID));
    RTRY(n->out.ensure(rows * NOUT)); RTRY(n->dO.ensure(rows * NOUT));
    n->cap_rows = rows;
    return DNSMC_OK;
}

// dW (M=nout x N=nin) = dZ^T H over rows, split over the rows; db = colsum(dZ)
int launch_gemm_tc(const GemmParams &G, dim3 grid, dnsmc_cvnet *n) {
    static int attr = 0;
    if (!attr) {
        CK(cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, GT_SMEM));
        attr = 1;
    }
    dnsmc::note_launch();
    gemm_tc_kernel<<<grid, 128, GT_SMEM, n->stream>>>(G, n->status.p);
    CK(cudaGetLastError());
    return DNSMC_OK;
}

int weight_grad(dnsmc_cvnet *n, const bf16 *dZ, int nout, const bf16 *H, int nin, long long rows, long long offW,
                long long offB) {
    const int splits = (int)std::min<long long>(64, std::max<long long>(1, rows / 256));
    const int klen = (int)(((rows + splits - 1) / splits + GT_K - 1) / GT_K * GT_K);
    RTRY(n->part.ensure((size_t)splits * nout * nin));
    GemmParams G{};
    G.M = nout; G.N = nin; G.K = (int)rows; G.klen = klen;
    G.A = dZ; G.a_sm = 1; G.a_sk = nout;
    G.B = H; G.b_sk = nin; G.b_sn = 1;
    G.C = n->part.p;
    RTRY(launch_gemm_tc(G, dim3((nout + 127) / 128, (nin + 127) / 128, splits), n));
    dnsmc::note_launch();
    reduce_splits_kernel<<<grid1((long long)nout * nin, 256), 256, 0, n->stream>>>(n->part.p, splits,
                                                                                   (long long)nout * nin,
                                                                                   n->grad.p + offW);
    CK(cudaGetLastError());
    dnsmc::note_launch();
    colsum_kernel<<<nout, 256, 0, n->stream>>>(dZ, rows, nout, n->grad.p + offB);
    CK(cudaGetLastError());
    return DNSMC_OK;
}

// dZprev (rows x nin) = (dZ W) * gelu'(Zprev)
int input_grad(dnsmc_cvnet *n, const bf16 *dZ, int nout, long long woff, int nin, long long rows, const float *Zprev,
               bf16 *dZprev) {
    GemmParams G{};
    G.M = (int)rows; G.N = nin; G.K = nout; G.klen = nout;
    G.A = dZ; G.a_sm = nout; G.a_sk = 1;
    G.B = n->W.p + woff; G.b_sk = nin; G.b_sn = 1;
    G.Z = Zprev; G.D = dZprev;
    return launch_gemm_tc(G, dim3((unsigned)((rows + 127) / 128), (nin + 127) / 128, 1), n);
}

// forward + loss + backward on `rows` rows (nvalid real) of X/lab through idx
int fwd_bwd(dnsmc_cvnet *n, const bf16 *X, const float *lab, int G, const int *idx, long long rows, long long nvalid,
            double loss[3]) {
    RTRY(ensure_work(n, rows));
    TcParams F{};
    F.rows = rows; F.X = X; F.idx = idx; F.nvalid = nvalid; F.out = n->out.p;
    F.H0 = n->H0.p; F.Z1 = n->Z1.p; F.Z2 = n->Z2.p; F.Z3 = n->Z3.p; F.H1 = n->H1.p; F.H2 = n->H2.p; F.H3 = n->H3.p;
    RTRY(launch_forward_tc(F, n, n->stream));
    LossParams L{};
    L.rows = rows; L.nvalid = nvalid; L.G = G; L.out = n->out.p; L.lab = lab; L.idx = idx;
    L.Sbeta = n->Sbeta; L.Sv = n->Sv; L.Sc = n->Sc; L.ridge = n->cfg.ridge; L.dout = n->dO.p;
    const int lblocks = grid1(rows, 256);
    RTRY(n->lpart.ensure((size_t)lblocks * 3));
    L.part = n->lpart.p;
    dnsmc::note_launch();
    loss_kernel<<<lblocks, 256, 0, n->stream>>>(L);
    CK(cudaGetLastError());
    RTRY(weight_grad(n, n->dO.p, NOUT, n->H3.p, HID, rows, OFF_W4, OFF_B4));
    RTRY(input_grad(n, n->dO.p, NOUT, WOFF_4, HID, rows, n->Z3.p, n->dZ3.p));
    RTRY(weight_grad(n, n->dZ3.p, HID, n->H2.p, HID, rows, OFF_W3, OFF_B3));
    RTRY(input_grad(n, n->dZ3.p, HID, WOFF_3, HID, rows, n->Z2.p, n->dZ2.p));
    RTRY(weight_grad(n, n->dZ2.p, HID, n->H1.p, HID, rows, OFF_W2, OFF_B2));
    RTRY(input_grad(n, n->dZ2.p, HID, WOFF_2, HID, rows, n->Z1.p, n->dZ1.p));
    RTRY(weight_grad(n, n->dZ1.p, HID, n->H0.p, K0, rows, OFF_W1, OFF_B1));
    if (loss) {
        std::vector<double> h((size_t)lblocks * 3);
        CK(cudaMemcpyAsync(h.data(), n->lpart.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, n->stream));
        CK(cudaStreamSynchronize(n->stream));
        loss[0] = loss[1] = loss[2] = 0.0;
        for (int b = 0; b < lblocks; ++b)
            for (int q = 0; q < 3; ++q) loss[q] += h[(size_t)b * 3 + q];
    }
    return DNSMC_OK;
}

int adam_step(dnsmc_cvnet *n) {
    n->step += 1;
    const float c1 = 1.0f - powf(n->cfg.adam_beta1, (float)n->step);
    const float c2 = 1.0f - powf(n->cfg.adam_beta2, (float)n->step);
    dnsmc::note_launch();
    adam_kernel<<<grid1(NPARAM, 256), 256, 0, n->stream>>>(n->P.p, n->grad.p, n->m.p, n->v.p, n->W.p, NPARAM,
                                                            n->cfg.lr, n->cfg.adam_beta1, n->cfg.adam_beta2,
                                                            n->cfg.adam_eps, c1, c2);
    CK(cudaGetLastError());
    dnsmc::note_launch();
    weights_to_bf16_kernel<<<grid1(NWEIGHT, 256), 256, 0, n->stream>>>(n->P.p, n->W.p);
    CK(cudaGetLastError());
    return DNSMC_OK;
}

int feature_params(dnsmc_cvnet *n, const SolverView &v, FeatParams *out) {
    FeatParams &F = *out;
    F = FeatParams{};
    F.nw = v.imax; F.na = v.jmax; F.nb = v.kmax; F.mode = v.mode;
    F.fT = v.fieldT; F.fTX = v.fieldTX; F.fw = v.fw; F.field_stride = v.field_stride;
    F.ew0 = v.i0; F.ea0 = v.j0; F.eb0 = v.k0;
    F.niR = v.i1 - v.i0; F.njR = v.j1 - v.j0; F.nkR = v.k1 - v.k0;
    F.region_cells = v.region_cells; F.nfields = v.nfields;
    F.Tc = n->cfg.T_center; F.Tis = 1.0f / n->cfg.T_scale;
    F.Xc = n->cfg.x_center; F.Xis = 1.0f / n->cfg.x_scale;
    if ((v.mode == MODE_TX && !v.fieldTX) || (v.mode != MODE_TX && !v.fieldT)) return state_fail("solver has no fields");
    return DNSMC_OK;
}

int features_for(dnsmc_cvnet *n, const SolverView &v, bf16 *out, cudaStream_t st) {
    FeatParams F{};
    F.nw = v.imax; F.na = v.jmax; F.nb = v.kmax; F.mode = v.mode;
    F.fT = v.fieldT; F.fTX = v.fieldTX; F.fw = v.fw; F.field_stride = v.field_stride;
    F.ew0 = v.i0; F.ea0 = v.j0; F.eb0 = v.k0;
    F.niR = v.i1 - v.i0; F.njR = v.j1 - v.j0; F.nkR = v.k1 - v.k0;
    F.region_cells = v.region_cells; F.nfields = v.nfields;
    F.Tc = n->cfg.T_center; F.Tis = 1.0f / n->cfg.T_scale;
    F.Xc = n->cfg.x_center; F.Xis = 1.0f / n->cfg.x_scale;
    F.out = out;
    if ((v.mode == MODE_TX && !v.fieldTX) || (v.mode != MODE_TX && !v.fieldT)) return state_fail("solver has no fields");
    dnsmc::note_launch();
    features_kernel<<<grid1((long long)v.nfields * v.region_cells, 128), 128, 0, st>>>(F);
    CK(cudaGetLastError());
    return DNSMC_OK;
}

int init_params(dnsmc_cvnet *n) {
    // He-style uniform init for hidden layers; zero output layer so the
    // untrained network is the plain control variate with uniform rays
    std::vector<float> h(NPARAM, 0.0f);
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    auto fill = [&](long long off, int rows, int cols, int fan_in) {
        const float a = sqrtf(6.0f / (float)fan_in);
        for (int r = 0; r < rows; ++r)
            for (int c = 0; c < cols; ++c) h[off + (long long)r * cols + c] = a * U(n->rng);
    };
    fill(OFF_W1, HID, K0, NFEAT);
    for (int r = 0; r < HID; ++r)
        for (int c = NFEAT; c < K0; ++c) h[OFF_W1 + (long long)r * K0 + c] = 0.0f;
    fill(OFF_W2, HID, HID, HID);
    fill(OFF_W3, HID, HID, HID);
    CK(cudaMemcpy(n->P.p, h.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemset(n->m.p, 0, NPARAM * sizeof(float)));
    CK(cudaMemset(n->v.p, 0, NPARAM * sizeof(float)));
    dnsmc::note_launch();
    weights_to_bf16_kernel<<<grid1(NWEIGHT, 256), 256, 0, n->stream>>>(n->P.p, n->W.p);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(n->stream));
    n->step = 0;
    return DNSMC_OK;
}

}  // namespace

extern "C" {

void dnsmc_cvnet_default_config(dnsmc_cvnet_config *c) {
    if (!c) return;
    memset(c, 0, sizeof *c);
    c->n_groups = 8;
    c->T_center = 1400.0f; c->T_scale = 1100.0f;
    c->x_center = 0.15f; c->x_scale = 0.15f;
    c->lr = 1e-3f; c->adam_beta1 = 0.9f; c->adam_beta2 = 0.999f; c->adam_eps = 1e-8f;
    c->ridge = 0.01f;
    c->batch = 4096;
    c->seed = 1;
}

int dnsmc_cvnet_create(const dnsmc_cvnet_config *cfg, dnsmc_cvnet **out) {
    if (!cfg || !out) return arg_fail("null argument");
    *out = nullptr;
    if (cfg->n_groups < 1 || cfg->n_groups > MAXG) return arg_fail("n_groups must be 1..16");
    if (!(cfg->T_scale > 0) || !(cfg->x_scale > 0)) return arg_fail("feature scales must be > 0");
    if (cfg->batch < 128 || cfg->batch % 128) return arg_fail("batch must be a positive multiple of 128");
    if (!(cfg->lr > 0) || !(cfg->ridge >= 0)) return arg_fail("bad lr or ridge");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) return report_error(DNSMC_ERR_NODEVICE, "no CUDA device");
    dnsmc_cvnet *n = new dnsmc_cvnet();
    n->cfg = *cfg;
    n->rng.seed(cfg->seed);
    int rc = DNSMC_OK;
    if ((e = cudaGetDevice(&n->device)) != cudaSuccess) rc = cuda_fail("cudaGetDevice", e);
    if (!rc && (e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking)) != cudaSuccess)
        rc = cuda_fail("cudaStreamCreate", e);
    if (!rc) rc = n->P.ensure(NPARAM);
    if (!rc) rc = n->grad.ensure(NPARAM);
    if (!rc) rc = n->m.ensure(NPARAM);
    if (!rc) rc = n->v.ensure(NPARAM);
    if (!rc) rc = n->W.ensure(2 * NWEIGHT);  // row-major and tensor-core order
    if (!rc) rc = n->status.ensure(1);
    if (!rc && (e = cudaMemset(n->status.p, 0, sizeof(unsigned int))) != cudaSuccess) rc = cuda_fail("cudaMemset", e);
    if (!rc) rc = init_params(n);
    if (rc) { delete n; return rc; }
    *out = n;
    return DNSMC_OK;
}

int dnsmc_cvnet_destroy(dnsmc_cvnet *n) {
    if (!n) return DNSMC_OK;
    cudaSetDevice(n->device);
    delete n;
    return DNSMC_OK;
}

long long dnsmc_cvnet_param_count(void) { return NPARAM; }

int dnsmc_cvnet_get_params(dnsmc_cvnet *n, float *params, float *scales) {
    if (!n) return arg_fail("null network");
    RTRY(set_dev(n));
    CK(cudaStreamSynchronize(n->stream));
    if (params) CK(cudaMemcpy(params, n->P.p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    if (scales) { scales[0] = n->Sbeta; scales[1] = n->Sv; scales[2] = n->Sc; }
    return DNSMC_OK;
}

int dnsmc_cvnet_set_params(dnsmc_cvnet *n, const float *params, const float *scales) {
    if (!n) return arg_fail("null network");
    RTRY(set_dev(n));
    CK(cudaStreamSynchronize(n->stream));
    if (params) {
        for (long long e = 0; e < NPARAM; ++e)
            if (!std::isfinite(params[e])) return arg_fail("parameters must be finite");
        CK(cudaMemcpy(n->P.p, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
        CK(cudaMemset(n->m.p, 0, NPARAM * sizeof(float)));
        CK(cudaMemset(n->v.p, 0, NPARAM * sizeof(float)));
        n->step = 0;
        dnsmc::note_launch();
        weights_to_bf16_kernel<<<grid1(NWEIGHT, 256), 256, 0, n->stream>>>(n->P.p, n->W.p);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(n->stream));
    }
    if (scales) {
        if (!(scales[0] > 0) || !(scales[1] > 0) || !(scales[2] > 0)) return arg_fail("label scales must be > 0");
        n->Sbeta = scales[0]; n->Sv = scales[1]; n->Sc = scales[2];
    }
    return DNSMC_OK;
}

int dnsmc_cvnet_save(dnsmc_cvnet *n, const char *path) {
    if (!n || !path) return arg_fail("null argument");
    std::vector<float> h(NPARAM);
    float sc[3];
    RTRY(dnsmc_cvnet_get_params(n, h.data(), sc));
    FILE *f = fopen(path, "wb");
    if (!f) return report_error(DNSMC_ERR_IO, "cannot open the network file for writing");
    const char magic[8] = {'D', 'N', 'S', 'M', 'C', 'N', 'N', '1'};
    const long long np = NPARAM;
    bool ok = fwrite(magic, 1, 8, f) == 8 && fwrite(&n->cfg, sizeof n->cfg, 1, f) == 1 &&
              fwrite(sc, sizeof(float), 3, f) == 3 && fwrite(&np, sizeof np, 1, f) == 1 &&
              fwrite(h.data(), sizeof(float), NPARAM, f) == (size_t)NPARAM;
    ok = (fclose(f) == 0) && ok;
    return ok ? DNSMC_OK : report_error(DNSMC_ERR_IO, "short write of the network file");
}

int dnsmc_cvnet_load(const char *path, dnsmc_cvnet **out) {
    if (!path || !out) return arg_fail("null argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return report_error(DNSMC_ERR_IO, "cannot open the network file");
    char magic[8];
    dnsmc_cvnet_config cfg;
    float sc[3];
    long long np = 0;
    std::vector<float> h(NPARAM);
    bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "DNSMCNN1", 8) == 0 && fread(&cfg, sizeof cfg, 1, f) == 1 &&
              fread(sc, sizeof(float), 3, f) == 3 && fread(&np, sizeof np, 1, f) == 1 && np == NPARAM &&
              fread(h.data(), sizeof(float), NPARAM, f) == (size_t)NPARAM;
    fclose(f);
    if (!ok) return report_error(DNSMC_ERR_IO, "not a network file of this version");
    dnsmc_cvnet *n = nullptr;
    RTRY(dnsmc_cvnet_create(&cfg, &n));
    int rc = dnsmc_cvnet_set_params(n, h.data(), (sc[0] > 0 && sc[1] > 0 && sc[2] > 0) ? sc : nullptr);
    if (rc) { dnsmc_cvnet_destroy(n); return rc; }
    *out = n;
    return DNSMC_OK;
}

int dnsmc_cvnet_features(dnsmc_cvnet *n, dnsmc_solver *s, float *host) {
    if (!n || !s || !host) return arg_fail("null argument");
    SolverView v;
    RTRY(solver_view(s, &v));
    if (v.device != n->device) return arg_fail("network and solver live on different devices");
    const long long rows = (long long)v.nfields * v.region_cells;
    RTRY(n->iX.ensure((size_t)rows * K0));
    RTRY(features_for(n, v, n->iX.p, (cudaStream_t)v.stream));
    std::vector<bf16> h((size_t)rows * K0);
    CK(cudaStreamSynchronize((cudaStream_t)v.stream));
    CK(cudaMemcpy(h.data(), n->iX.p, h.size() * sizeof(bf16), cudaMemcpyDeviceToHost));
    for (long long r = 0; r < rows; ++r)
        for (int q = 0; q < NFEAT; ++q) host[r * NFEAT + q] = __bfloat162float(h[(size_t)(r * K0 + q)]);
    return DNSMC_OK;
}

int dnsmc_cvnet_add_training_data(dnsmc_cvnet *n, dnsmc_solver *s) {
    if (!n || !s) return arg_fail("null argument");
    SolverView v;
    RTRY(solver_view(s, &v));
    if (v.device != n->device) return arg_fail("network and solver live on different devices");
    RTRY(dnsmc_wait(s, 0.0));
    if (!v.solved || !v.moments) return state_fail("training data needs a solve with control_variate and cv_moments set");
    if (v.last_groups > n->cfg.n_groups) return arg_fail("the solve has more band groups than the network");
    if (n->nrows > 0 && v.last_groups != n->dG) return arg_fail("band groups differ from the data already added");
    const int G = v.last_groups;
    const long long rows = (long long)v.nfields * v.region_cells;
    const long long total = n->nrows + rows;
    cudaStream_t st = (cudaStream_t)v.stream;
    // grow the dataset (copy the old rows)
    if ((size_t)(total * K0) > n->dX.n || (size_t)(total * G * NLAB) > n->dlab.n) {
        NBuf<bf16> nx;
        NBuf<float> nl;
        const long long cap = std::max(total, n->nrows * 2);
        RTRY(nx.ensure((size_t)cap * K0));
        RTRY(nl.ensure((size_t)cap * G * NLAB));
        if (n->nrows) {
            CK(cudaMemcpyAsync(nx.p, n->dX.p, (size_t)n->nrows * K0 * sizeof(bf16), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(nl.p, n->dlab.p, (size_t)n->nrows * G * NLAB * sizeof(float), cudaMemcpyDeviceToDevice, st));
        }
        CK(cudaStreamSynchronize(st));
        n->dX.release(); n->dlab.release();
        n->dX = nx; n->dlab = nl;
        nx.p = nullptr; nl.p = nullptr;
    }
    RTRY(features_for(n, v, n->dX.p + n->nrows * K0, st));
    LabelParams L{};
    L.nfields = v.nfields; L.G = G; L.niR = v.i1 - v.i0; L.njR = v.j1 - v.j0; L.nkR = v.k1 - v.k0;
    L.tile_a = v.tile_a; L.tile_b = v.tile_b; L.npa = v.npa; L.npb = v.npb; L.n_packets = v.n_packets;
    L.region_cells = v.region_cells; L.moments = v.moments; L.varg = v.varg; L.steps = v.item_steps;
    L.rays = v.rays; L.rays_item = v.rays_item; L.rays_gstride = v.rays_gstride;
    L.lab = n->dlab.p + n->nrows * G * NLAB;
    dnsmc::note_launch();
    labels_kernel<<<grid1(rows, 128), 128, 0, st>>>(L);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    if (!(n->Sbeta > 0)) {
        // label scales from the first data: mean V(1,-1), mean v, mean c
        std::vector<float> h((size_t)rows * G * NLAB);
        CK(cudaMemcpy(h.data(), L.lab, h.size() * sizeof(float), cudaMemcpyDeviceToHost));
        double sb = 0, sv = 0, sc = 0;
        long long nb = 0, nv = 0, nc = 0;
        for (long long q = 0; q < rows * G; ++q) {
            const float *y = &h[(size_t)q * NLAB];
            const double V0 = (double)y[0] - 2.0 * y[3] + 2.0 * y[4] + y[1] - 2.0 * y[5] + y[2];
            if (y[0] > 0 || y[1] > 0) { sb += V0; ++nb; }
            if (y[6] > 0) { sv += y[6]; ++nv; }
            if (y[7] > 0) { sc += y[7]; ++nc; }
        }
        n->Sbeta = nb && sb > 0 ? (float)(sb / nb) : 1.0f;
        n->Sv = nv && sv > 0 ? (float)(sv / nv) : 1.0f;
        n->Sc = nc && sc > 0 ? (float)(sc / nc) : 1.0f;
    }
    n->nrows = total;
    n->dG = G;
    return DNSMC_OK;
}

int dnsmc_cvnet_clear_training_data(dnsmc_cvnet *n) {
    if (!n) return arg_fail("null network");
    n->nrows = 0;
    return DNSMC_OK;
}

long long dnsmc_cvnet_training_rows(const dnsmc_cvnet *n) { return n ? n->nrows : -1; }

int dnsmc_cvnet_train(dnsmc_cvnet *n, int epochs, double *loss) {
    if (!n) return arg_fail("null network");
    if (epochs < 1) return arg_fail("epochs must be >= 1");
    if (n->nrows < 1) return state_fail("no training data");
    RTRY(set_dev(n));
    const long long B = n->cfg.batch;
    RTRY(ensure_work(n, B));
    std::vector<int> perm((size_t)n->nrows);
    double acc[3] = {0, 0, 0};
    long long nb = 0;
    for (int ep = 0; ep < epochs; ++ep) {
        for (long long i = 0; i < n->nrows; ++i) perm[(size_t)i] = (int)i;
        std::shuffle(perm.begin(), perm.end(), n->rng);
        for (long long b0 = 0; b0 < n->nrows; b0 += B) {
            const long long nv = std::min(B, n->nrows - b0);
            CK(cudaMemcpyAsync(n->idx.p, perm.data() + b0, nv * sizeof(int), cudaMemcpyHostToDevice, n->stream));
            double l[3];
            const bool last = (ep == epochs - 1);
            RTRY(fwd_bwd(n, n->dX.p, n->dlab.p, n->dG, n->idx.p, B, nv, last ? l : nullptr));
            RTRY(adam_step(n));
            if (last) {
                for (int q = 0; q < 3; ++q) acc[q] += l[q];
                nb += nv;
            }
        }
    }
    CK(cudaStreamSynchronize(n->stream));
    if (loss) {
        for (int q = 0; q < 3; ++q) loss[q + 1] = nb ? acc[q] / nb : 0.0;
        loss[0] = loss[1] + loss[2] + loss[3];
    }
    return DNSMC_OK;
}

int dnsmc_cvnet_eval(dnsmc_cvnet *n, const float *features, long long rows, float *out) {
    if (!n || !features || !out || rows < 1) return arg_fail("bad argument");
    RTRY(set_dev(n));
    std::vector<bf16> h((size_t)rows * K0);
    for (long long r = 0; r < rows; ++r)
        for (int q = 0; q < K0; ++q)
            h[(size_t)(r * K0 + q)] = __float2bfloat16(q < NFEAT ? features[r * NFEAT + q] : 0.0f);
    RTRY(n->iX.ensure((size_t)rows * K0));
    RTRY(n->iout.ensure((size_t)rows * NOUT));
    CK(cudaMemcpyAsync(n->iX.p, h.data(), h.size() * sizeof(bf16), cudaMemcpyHostToDevice, n->stream));
    TcParams F{};
    F.rows = rows; F.X = n->iX.p; F.nvalid = rows; F.out = n->iout.p;
    RTRY(launch_forward_tc(F, n, n->stream));
    CK(cudaMemcpyAsync(out, n->iout.p, (size_t)rows * NOUT * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    unsigned int st = 0;
    CK(cudaMemcpyAsync(&st, n->status.p, sizeof st, cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    if (st) return report_error(DNSMC_ERR_TIMEOUT, "network forward: a bounded wait for the tensor cores ran out");
    return DNSMC_OK;
}

int dnsmc_cvnet_gradient(dnsmc_cvnet *n, const float *features, const float *labels, int n_groups, long long rows,
                         float *grad, double *loss) {
    if (!n || !features || !labels || !grad || rows < 1) return arg_fail("bad argument");
    if (n_groups < 1 || n_groups > n->cfg.n_groups) return arg_fail("bad n_groups");
    if (!(n->Sbeta > 0) || !(n->Sv > 0) || !(n->Sc > 0)) return state_fail("label scales unset");
    RTRY(set_dev(n));
    const long long R = (rows + 127) / 128 * 128;
    std::vector<bf16> h((size_t)R * K0, __float2bfloat16(0.0f));
    for (long long r = 0; r < rows; ++r)
        for (int q = 0; q < NFEAT; ++q) h[(size_t)(r * K0 + q)] = __float2bfloat16(features[r * NFEAT + q]);
    NBuf<bf16> x;
    NBuf<float> lab;
    RTRY(x.ensure((size_t)R * K0));
    RTRY(lab.ensure((size_t)rows * n_groups * NLAB));
    CK(cudaMemcpy(x.p, h.data(), h.size() * sizeof(bf16), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(lab.p, labels, (size_t)rows * n_groups * NLAB * sizeof(float), cudaMemcpyHostToDevice));
    double l[3];
    int rc = fwd_bwd(n, x.p, lab.p, n_groups, nullptr, R, rows, l);
    if (!rc) {
        cudaError_t e = cudaMemcpy(grad, n->grad.p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail("cudaMemcpy", e);
    }
    x.release();
    lab.release();
    if (!rc && loss) {
        for (int q = 0; q < 3; ++q) loss[q + 1] = l[q] / rows;
        loss[0] = loss[1] + loss[2] + loss[3];
    }
    return rc;
}

int dnsmc_cvnet_apply(dnsmc_cvnet *n, dnsmc_solver *s, int flags, int mean_rays, int min_rays, int max_rays) {
    if (!n || !s) return arg_fail("null argument");
    if (!(flags & (DNSMC_CVNET_BETA | DNSMC_CVNET_RAYS))) return arg_fail("flags select nothing");
    if (!(n->Sv > 0) || !(n->Sc > 0)) return state_fail("untrained network: label scales unset");
    SolverView v;
    RTRY(solver_view(s, &v));
    if (v.device != n->device) return arg_fail("network and solver live on different devices");
    if (v.n_groups > n->cfg.n_groups) return arg_fail("the solver has more band groups than the network");
    const int B = v.sampler == DNSMC_SAMPLER_RQMC ? v.nvar : 1;
    if (flags & DNSMC_CVNET_RAYS) {
        if (min_rays < std::max(2, B) || mean_rays < min_rays || max_rays < mean_rays)
            return arg_fail("ray bounds must satisfy max(2, nvar) <= min_rays <= mean_rays <= max_rays");
        if (mean_rays % B || min_rays % B || max_rays % B) return arg_fail("RQMC: ray bounds must be multiples of nvar");
    }
    const int G = v.n_groups;
    const long long rows = (long long)v.nfields * v.region_cells;
    cudaStream_t st = (cudaStream_t)v.stream;
    float2 *beta = nullptr;
    long long nbeta = 0;
    if (flags & DNSMC_CVNET_BETA) RTRY(solver_beta_device(s, &beta, &nbeta));
    int *rays = nullptr;
    if (flags & DNSMC_CVNET_RAYS) RTRY(solver_rays_device(s, G, &rays));
    RTRY(n->vc.ensure((size_t)rows * G));
    // features, the four layers on the tensor cores and the coefficient
    // epilogue in one kernel: neither features nor outputs go through memory
    TcParams F{};
    F.rows = rows;
    F.fused_features = 1;
    RTRY(feature_params(n, v, &F.feat));
    F.fused_apply = 1;
    F.apply.rows = rows; F.apply.G = G; F.apply.Sv = n->Sv; F.apply.Sc = n->Sc; F.apply.beta = beta;
    F.apply.vc = n->vc.p; F.apply.region_cells = v.region_cells;
    // the network's weights are written on its own stream
    CK(cudaStreamSynchronize(n->stream));
    RTRY(launch_forward_tc(F, n, st));
    if (flags & DNSMC_CVNET_RAYS) {
        const long long items = (long long)G * v.n_packets;
        RTRY(n->wgt.ensure((size_t)items));
        RTRY(n->cost.ensure((size_t)items));
        RTRY(n->lam.ensure(1));
        RTRY(n->lam_part.ensure(kScaleBlocks));
        RTRY(n->lam_done.ensure(1));
        CK(cudaMemsetAsync(n->lam_done.p, 0, sizeof(unsigned int), st));
        AllocParams P{};
        P.nfields = v.nfields; P.G = G; P.n_packets = v.n_packets; P.npa = v.npa; P.npb = v.npb;
        P.tile_a = v.tile_a; P.tile_b = v.tile_b; P.njR = v.j1 - v.j0; P.nkR = v.k1 - v.k0;
        P.region_cells = v.region_cells; P.vc = n->vc.p; P.wgt = n->wgt.p; P.cost = n->cost.p;
        dnsmc::note_launch();
        alloc_weights_kernel<<<grid1(items * 32, 256), 256, 0, st>>>(P);
        CK(cudaGetLastError());
        dnsmc::note_launch();
        alloc_scale_kernel<<<kScaleBlocks, kScaleThreads, 0, st>>>(n->wgt.p, n->cost.p, items, (float)mean_rays,
                                                                    n->lam.p, n->lam_part.p, n->lam_done.p);
        CK(cudaGetLastError());
        dnsmc::note_launch();
        alloc_rays_kernel<<<grid1(items, 256), 256, 0, st>>>(n->wgt.p, items, n->lam.p, B, min_rays, max_rays, rays);
        CK(cudaGetLastError());
    }
    return DNSMC_OK;
}

}  // extern "C"
