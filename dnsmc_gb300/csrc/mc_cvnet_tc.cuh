// mc_cvnet_tc.cuh -- the network's forward pass and the backward pass's
// GEMMs on the fifth-generation tensor cores (tcgen05) with the accumulators
// in tensor memory.  Included by mc_cvnet.cu (it uses that file's constants,
// GELU and feature row).  The forward pass:
//
// One CTA per SM, persistent over 128-row tiles; TC_WG warpgroups per CTA,
// each with its own tile in flight so that one warpgroup's epilogue (bias,
// GELU, bf16 packing) runs while the tensor core works on the others' layers
// (three: 0.71 ms for the 2.1M rows of a 128^3 field, two: 0.80 ms).
// Per tile and warpgroup:
//
//   features of its 128 rows (feature_row, one row per thread) or rows of a
//   bf16 feature array -> shared memory, as the A operand of layer 1;
//   for each layer: one elected thread issues tcgen05.mma (M = 128, N = 128
//   or 64, K = 16 per instruction, bf16 x bf16 -> f32) from the A tile and
//   the layer's weights (B) in shared memory into the warpgroup's 128
//   tensor-memory columns, and commits to the warpgroup's mbarrier; the
//   warpgroup waits (bounded), reads its rows back with tcgen05.ld (thread t
//   holds row t), adds the bias and applies GELU, and writes the bf16
//   activations into the A tile for the next layer;
//   the output layer's 64 values per row go to the output rows, or through
//   the coefficient epilogue (beta, and the variance and cost heads) that
//   dnsmc_cvnet_apply needs, without an output array in between.
//
// Operand layout in shared memory: the K-major layout without swizzle of
// the tcgen05 matrix descriptors -- core matrices of 8 rows x 16 bytes (8
// bf16 along K), a row's 8-element K chunks `chunk` apart:
//   element (row, k) at (k / 8) * rows * 16 + row * 16 + (k % 8) * 2 bytes,
// so the descriptor's stride between 8-row groups is 128 bytes and between
// the two K chunks of one instruction rows * 16 bytes.  The weights are
// kept in that order in global memory (weights_to_bf16_kernel writes it) and
// arrive by one bulk copy (cp.async.bulk) per CTA.
#pragma once

namespace {

constexpr int TC_WG = 3;                 // warpgroups (tiles in flight) per CTA
constexpr int TC_THREADS = 128 * TC_WG;
// tensor-memory columns of the CTA: 128 per warpgroup, allocated as a power of two
constexpr uint32_t TC_TMEM_COLS = TC_WG * 128 <= 128 ? 128 : (TC_WG * 128 <= 256 ? 256 : 512);
static_assert(TC_WG * 128 <= 512, "tensor memory holds 512 columns");
constexpr int TC_TILE = 128;             // rows per tile (the MMA's M)
// shared-memory map (bytes)
constexpr uint32_t TC_W1 = 0;                                  // [K0/8][HID][8] bf16
constexpr uint32_t TC_W2 = TC_W1 + HID * K0 * 2;               // [HID/8][HID][8]
constexpr uint32_t TC_W3 = TC_W2 + HID * HID * 2;
constexpr uint32_t TC_W4 = TC_W3 + HID * HID * 2;              // [HID/8][NOUT][8]
constexpr uint32_t TC_WBYTES = TC_W4 + NOUT * HID * 2;         // 102400
constexpr uint32_t TC_BIAS = TC_WBYTES;                        // (3 HID + NOUT) floats
constexpr uint32_t TC_ACT = (TC_BIAS + (3 * HID + NOUT) * 4 + 1023) / 1024 * 1024;
constexpr uint32_t TC_ACT_BYTES = TC_TILE * HID * 2;           // one A tile: [HID/8][128][8] bf16
constexpr uint32_t TC_BAR = TC_ACT + TC_WG * TC_ACT_BYTES;     // mbarriers and the TMEM address
constexpr uint32_t TC_SMEM = TC_BAR + 64;
static_assert(TC_WBYTES == NWEIGHT * 2, "weight copy size");
static_assert(TC_SMEM <= 227 * 1024, "shared memory of the tensor-memory forward");
// bounded polls of an mbarrier before the kernel records a time-out
constexpr int TC_POLLS = 1 << 22;

// Index of weight element (row n, column k) of an N x K matrix in the
// tensor-core order [K/8][N][8].
__host__ __device__ __forceinline__ long long tc_index(int n, int k, int N) {
    return (long long)(k >> 3) * N * 8 + (long long)n * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of tcgen05 (K-major, no swizzle): start
// address, leading-dimension byte offset (between the two K core matrices
// of an instruction), stride-dimension byte offset (between 8-row groups),
// each encoded >> 4; bits 46-47 = 1 (descriptor version of this
// architecture); base offset, LBO mode and swizzle mode 0.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16: D f32 (bits 4-5 = 1),
// A and B bf16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(bar))
                 : "memory");
}

__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t b = tc_smem(bar);
    for (int it = 0; it < TC_POLLS; ++it) {
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

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_bar(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

// 32 consecutive f32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct TcParams {
    long long rows;
    int fused_features;       // 1: features of the solver's region (feat); 0: bf16 rows of X
    FeatParams feat;
    const bf16 *X;            // [*][K0] feature rows
    const int *idx;           // row r reads X[idx[r]] (null: X[r]); rows >= nvalid read zeros
    long long nvalid;
    // training saves (all null at inference): the layer-1 input rows, the
    // pre-activations Z and the bf16 activations H of the hidden layers
    bf16 *H0;                 // [rows][K0]
    float *Z1, *Z2, *Z3;      // [rows][HID]
    bf16 *H1, *H2, *H3;       // [rows][HID]
    const bf16 *Wtc;          // the four weight matrices in tensor-core order
    const float *P;           // FP32 master parameters (biases)
    float *out;               // [rows][NOUT] (fused_apply 0)
    int fused_apply;          // 1: the coefficient epilogue below instead of out
    ApplyParams apply;
    unsigned int *status;     // bit 1: a bounded wait ran out
};

// Layer of one tile: MMAs over K (K/16 instructions) from the A tile into
// the warpgroup's accumulator columns, committed to its barrier.
template <int K, int N>
__device__ __forceinline__ void tc_layer(uint32_t a_addr, uint32_t b_addr, uint32_t dtmem, uint64_t *bar) {
    constexpr uint32_t lbo_a = TC_TILE * 16, lbo_b = N * 16;
#pragma unroll
    for (int k = 0; k < K / 16; ++k) {
        const uint64_t da = tc_desc(a_addr + k * 2 * lbo_a, lbo_a, 128);
        const uint64_t db = tc_desc(b_addr + k * 2 * lbo_b, lbo_b, 128);
        tc_mma(dtmem, da, db, tc_idesc(TC_TILE, N), k > 0 ? 1u : 0u);
    }
    tc_commit(bar);
}

// Hidden-layer epilogue: the 128 accumulator columns of this thread's row,
// bias and GELU, packed to bf16 into the A tile (this row's 16-byte chunks);
// in training also the row's pre-activations (Zs) and activations (Hs).
__device__ __forceinline__ void tc_hidden(uint32_t tlane, const float *bias, unsigned char *act, int lt, float *Zs,
                                          bf16 *Hs) {
#pragma unroll
    for (int c = 0; c < HID / 32; ++c) {
        uint32_t v[32];
        tc_ld32(tlane + c * 32, v);
        uint32_t h[16];
        float z[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) z[q] = __uint_as_float(v[q]) + bias[c * 32 + q];
#pragma unroll
        for (int q = 0; q < 16; ++q) h[q] = pack_bf16(gelu(z[2 * q]), gelu(z[2 * q + 1]));
#pragma unroll
        for (int m = 0; m < 4; ++m)
            *reinterpret_cast<uint4 *>(act + (c * 4 + m) * (TC_TILE * 16) + lt * 16) =
                make_uint4(h[4 * m], h[4 * m + 1], h[4 * m + 2], h[4 * m + 3]);
        if (Zs) {
            float4 *zd = reinterpret_cast<float4 *>(Zs + c * 32);
#pragma unroll
            for (int m = 0; m < 8; ++m) zd[m] = make_float4(z[4 * m], z[4 * m + 1], z[4 * m + 2], z[4 * m + 3]);
            uint4 *hd = reinterpret_cast<uint4 *>(Hs + c * 32);
#pragma unroll
            for (int m = 0; m < 4; ++m) hd[m] = make_uint4(h[4 * m], h[4 * m + 1], h[4 * m + 2], h[4 * m + 3]);
        }
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1) mlp_tc_kernel(const TcParams F) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, wg = tid >> 7, lt = tid & 127, warp = tid >> 5;
    uint64_t *bar_w = reinterpret_cast<uint64_t *>(sm + TC_BAR);
    uint64_t *bar_m = bar_w + 1 + wg;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + TC_BAR + 32);
    float *bias = reinterpret_cast<float *>(sm + TC_BIAS);
    unsigned char *act = sm + TC_ACT + wg * TC_ACT_BYTES;
    const uint32_t act_a = tc_smem(act);
    const uint32_t w_a = tc_smem(sm);
    unsigned int err = 0;

    if (tid == 0) {
        for (int b = 0; b < 1 + TC_WG; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(bar_w + b)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int e = tid; e < HID; e += TC_THREADS) {
        bias[e] = F.P[OFF_B1 + e];
        bias[HID + e] = F.P[OFF_B2 + e];
        bias[2 * HID + e] = F.P[OFF_B3 + e];
    }
    for (int e = tid; e < NOUT; e += TC_THREADS) bias[3 * HID + e] = F.P[OFF_B4 + e];
    if (warp == 0) {  // the accumulators of all warpgroups: 128 columns each
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot + (uint32_t)(wg * 128);         // this warpgroup's columns, lane 0
    const uint32_t tlane = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's 32 lanes
    if (tid == 0) {  // the weights, in tensor-core order, by one bulk copy
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc_smem(bar_w)), "r"(TC_WBYTES)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         w_a),
                     "l"(F.Wtc), "r"(TC_WBYTES), "r"(tc_smem(bar_w))
                     : "memory");
    }
    if (!tc_wait(bar_w, 0)) err |= 2u;

    uint32_t ph = 0;
    const long long ntiles = (F.rows + TC_TILE - 1) / TC_TILE;
    const int bid = 1 + wg;  // this warpgroup's named barrier
    for (long long tile = (long long)blockIdx.x * TC_WG + wg; tile < ntiles; tile += (long long)gridDim.x * TC_WG) {
        const long long r = tile * TC_TILE + lt;
        const bool valid = r < F.rows;
        // ---- layer-1 input: this row's features, K0 / 8 chunks of 16 bytes
        uint32_t x[K0 / 2];
        if (!valid) {
#pragma unroll
            for (int q = 0; q < K0 / 2; ++q) x[q] = 0u;
        } else if (F.fused_features) {
            feature_row(F.feat, r, x);
        } else if (r >= F.nvalid) {
#pragma unroll
            for (int q = 0; q < K0 / 2; ++q) x[q] = 0u;
        } else {
            const long long sr = F.idx ? (long long)F.idx[r] : r;
            const uint4 *src = reinterpret_cast<const uint4 *>(F.X + sr * K0);
#pragma unroll
            for (int c = 0; c < K0 / 8; ++c) {
                const uint4 u = src[c];
                x[4 * c] = u.x; x[4 * c + 1] = u.y; x[4 * c + 2] = u.z; x[4 * c + 3] = u.w;
            }
        }
#pragma unroll
        for (int c = 0; c < K0 / 8; ++c)
            *reinterpret_cast<uint4 *>(act + c * (TC_TILE * 16) + lt * 16) =
                make_uint4(x[4 * c], x[4 * c + 1], x[4 * c + 2], x[4 * c + 3]);
        if (F.H0 && valid) {
            uint4 *hd = reinterpret_cast<uint4 *>(F.H0 + r * K0);
#pragma unroll
            for (int c = 0; c < K0 / 8; ++c) hd[c] = make_uint4(x[4 * c], x[4 * c + 1], x[4 * c + 2], x[4 * c + 3]);
        }
        // ---- four layers
#pragma unroll 1
        for (int layer = 0; layer < 4; ++layer) {
            tc_proxy_fence();  // the A tile's generic stores, visible to the tensor core
            tc_fence_before();
            tc_bar(bid);
            if (lt == 0) {
                tc_fence_after();
                if (layer == 0) tc_layer<K0, HID>(act_a, w_a + TC_W1, tmem, bar_m);
                else if (layer == 1) tc_layer<HID, HID>(act_a, w_a + TC_W2, tmem, bar_m);
                else if (layer == 2) tc_layer<HID, HID>(act_a, w_a + TC_W3, tmem, bar_m);
                else tc_layer<HID, NOUT>(act_a, w_a + TC_W4, tmem, bar_m);
            }
            if (!tc_wait(bar_m, ph)) err |= 2u;
            ph ^= 1u;
            tc_fence_after();
            if (layer < 3) {
                float *Zs = layer == 0 ? F.Z1 : (layer == 1 ? F.Z2 : F.Z3);
                bf16 *Hs = layer == 0 ? F.H1 : (layer == 1 ? F.H2 : F.H3);
                const bool save = Zs && valid;
                tc_hidden(tlane, bias + layer * HID, act, lt, save ? Zs + r * HID : nullptr,
                          save ? Hs + r * HID : nullptr);
                continue;
            }
            // ---- output layer: 64 values of this row
            uint32_t v0[32], v1[32];
            tc_ld32(tlane, v0);
            tc_ld32(tlane + 32, v1);
            if (!valid) break;
            float o[NOUT];
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                o[c] = __uint_as_float(v0[c]) + bias[3 * HID + c];
                o[32 + c] = __uint_as_float(v1[c]) + bias[3 * HID + 32 + c];
            }
            if (!F.fused_apply) {
                float4 *dst = reinterpret_cast<float4 *>(F.out + r * NOUT);
#pragma unroll
                for (int c = 0; c < NOUT / 4; ++c) dst[c] = make_float4(o[4 * c], o[4 * c + 1], o[4 * c + 2], o[4 * c + 3]);
            } else {
                const ApplyParams &A = F.apply;
                const long long f = r / A.region_cells, tc = r - f * A.region_cells;
#pragma unroll
                for (int g = 0; g < MAXG; ++g) {
                    if (g >= A.G) break;
                    const long long d = (f * A.G + g) * A.region_cells + tc;
                    if (A.beta) {
                        float ba = 1.0f + o[4 * g], bb = -1.0f + o[4 * g + 1];
                        if (!isfinite(ba) || !isfinite(bb)) { ba = 1.0f; bb = -1.0f; }
                        A.beta[d] = make_float2(ba, bb);
                    }
                    A.vc[d] = make_float2(A.Sv * expf(clampo(o[4 * g + 2])), A.Sc * expf(clampo(o[4 * g + 3])));
                }
            }
        }
    }
    if (err && F.status) atomicOr(F.status, err);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tslot), "r"(TC_TMEM_COLS)
                     : "memory");
    }
}


// ---------------------------------------------------------------------------
// Training GEMMs on tcgen05: C (M x N) = A (M x K) B (K x N) over the CTA's K
// range (blockIdx.z x klen), A(m, k) = A[m a_sm + k a_sk], B(k, n) =
// B[k b_sk + n b_sn], bf16 operands, f32 accumulator in tensor memory.  One
// CTA (one warpgroup) per 128 x Nt tile (Nt <= 128, a multiple of 16; rows of
// A beyond M read zeros); K in stages of 64 staged by plain loads into the
// descriptors' K-major layout; one elected thread issues the four MMAs of a
// stage and commits, the warpgroup waits (bounded) before the next stage.
// Epilogue (thread t = row t): f32 partials C[split][M][N], or D = bf16(acc x
// GELU'(Z)) (the input gradient of the previous layer).
// ---------------------------------------------------------------------------
constexpr int GT_K = 64;
constexpr int GT_SMEM = 64 * 1024;  // two 16 KB operand tiles; the size keeps at most 3 CTAs (384 TMEM columns) per SM

__global__ void __launch_bounds__(128) gemm_tc_kernel(const GemmParams G, unsigned int *status) {
    extern __shared__ __align__(1024) unsigned char gsm[];
    unsigned char *sA = gsm, *sB = gsm + 128 * GT_K * 2;
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * 128;
    const int nt = min(128, G.N - n0);
    const int ntp = (nt + 15) & ~15;
    const int kbeg = blockIdx.z * G.klen, kend = min(G.K, kbeg + G.klen);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(tc_smem(&tslot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t aA = tc_smem(sA), aB = tc_smem(sB);
    const bf16 zero = __float2bfloat16(0.0f);
    uint32_t ph = 0;
    unsigned int err = 0;
    for (int k0 = kbeg; k0 < kend; k0 += GT_K) {
        // A: 128 rows x 8 chunks of 8 along K
        for (int it = tid; it < 128 * (GT_K / 8); it += 128) {
            const int m = it & 127, c = it >> 7;
            const int gm = m0 + m, gk = k0 + 8 * c;
            __align__(16) bf16 v[8];
            if (gm < G.M && G.a_sk == 1 && gk + 8 <= kend) {
                *reinterpret_cast<uint4 *>(v) = *reinterpret_cast<const uint4 *>(G.A + (long long)gm * G.a_sm + gk);
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    v[e] = (gm < G.M && gk + e < kend) ? G.A[(long long)gm * G.a_sm + (long long)(gk + e) * G.a_sk] : zero;
            }
            *reinterpret_cast<uint4 *>(sA + c * (128 * 16) + m * 16) = *reinterpret_cast<const uint4 *>(v);
        }
        // B: ntp rows (n) x 8 chunks of 8 along K
        for (int it = tid; it < ntp * (GT_K / 8); it += 128) {
            const int n = it % ntp, c = it / ntp;
            const int gn = n0 + n, gk = k0 + 8 * c;
            __align__(16) bf16 v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e)
                v[e] = (n < nt && gk + e < kend) ? G.B[(long long)(gk + e) * G.b_sk + (long long)gn * G.b_sn] : zero;
            *reinterpret_cast<uint4 *>(sB + c * (ntp * 16) + n * 16) = *reinterpret_cast<const uint4 *>(v);
        }
        tc_proxy_fence();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int k = 0; k < GT_K / 16; ++k) {
                const uint64_t da = tc_desc(aA + k * 2 * (128 * 16), 128 * 16, 128);
                const uint64_t db = tc_desc(aB + k * 2 * (ntp * 16), ntp * 16, 128);
                tc_mma(tmem, da, db, tc_idesc(128, ntp), (k0 > kbeg || k > 0) ? 1u : 0u);
            }
            tc_commit(&bar);
        }
        if (!tc_wait(&bar, ph)) err |= DNSMC_STATUS_COPY_TIMEOUT;
        ph ^= 1u;
        tc_fence_after();
    }
    const int gm = m0 + tid;
    const bool any = kend > kbeg;
    for (int c = 0; c < (ntp + 31) / 32; ++c) {
        uint32_t v[32];
        tc_ld32(tlane + c * 32, v);
        if (gm >= G.M) continue;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const int n = c * 32 + q;
            if (n >= nt) break;
            const float a = any ? __uint_as_float(v[q]) : 0.0f;
            const long long o = (long long)gm * G.N + n0 + n;
            if (G.D) G.D[o] = __float2bfloat16(a * gelu_grad(G.Z[o]));
            else G.C[(long long)blockIdx.z * G.M * G.N + o] = a;
        }
    }
    if (err && status) atomicOr(status, err);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
    }
}
}  // namespace
