// mc_march_pair.cuh -- the march on the fine grid (the reference's
// kernel_fluid + march_ray, code/mc_gpu.cu:44-438), two cells per lane: the
// absorbing gas with black walls (march_pair_kernel), and the general medium
// with scattering particles and grey walls (march_gen_kernel).
//
// A packet here is 64 cells of one wall-normal plane: tile_a cells along j
// by tile_b = 64 / tile_a along k.  Lane l owns packet cells l and l + 32,
// which share their j index and lie 32 / tile_a rows apart in k.  Every ray
// of the packet shares one direction and one spectral sample, so the voxel
// walk (which face is crossed next, every segment length) is the same for
// all 64 cells: it is computed once per lane for two cells, and only the
// per-cell work (field gather, k and Ib lookups, attenuation, tallies) is
// done twice.  Every cell's arithmetic is the reference estimator's update
// written with explicit fmaf, and the host replay (oracle/mc_oracle.cpp)
// marches the same 64-cell packets, so it reproduces every cell bit for bit.
//
// march_gen_kernel is the same march for the general medium: absorption
// k + fv a_band and scattering fv s_band per cell; weighted delta tracking
// with a warp-shared decision (q = mean over the packet's live cells of
// fv s_band / majorant, summed by each lane over its cells in order and then
// across lanes; each cell's throughput is multiplied by p / q on a scatter
// and (1 - p) / (1 - q) otherwise, so every cell's expectation is that of
// ordinary delta tracking); Henyey-Greenstein directions; grey diffuse walls.
// Every direction change restarts the walk from the current point.
//
// Its translation units (mc_march_pair.cu, mc_march_gen.cu) are compiled
// with -fmad=false like the other march translation units.
#pragma once
#include "mc_march.cuh"

namespace dnsmc {

// Resident 256-thread blocks per SM of this march (2: up to 128 registers a
// thread; its two cells per lane carry twice the per-cell state).
#ifndef DNSMC_PAIR_MINB
#define DNSMC_PAIR_MINB 2
#endif
template <int MODE, bool TRACE, bool CV, bool MOM>
__global__ void __launch_bounds__(256, DNSMC_PAIR_MINB) march_pair_kernel(const MarchParams P) {
    typedef typename FieldT<MODE>::type VT;
    constexpr int C = kLaneCells;  // cells per lane
    static_assert(C % 2 == 0, "the attenuation goes through cell pairs");
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int tid = threadIdx.x;
    const int la = lane % P.tile_a, lb = lane / P.tile_a;
    const int hb = 32 / P.tile_a;  // k rows between a lane's two cells
    const int njR = P.ea1 - P.ea0, nkR = P.eb1 - P.eb0;
    const int plane = P.na * P.nb;
    unsigned long long my_rays = 0, my_steps = 0;
    unsigned int flags = 0;
    // dynamic shared memory (march_smem): this warp's copy of the current
    // ray's table slab (tabulated models); per-cell sums of the item as
    // float pairs (ray sum, sum of squares or of squared replicate means,
    // current replicate sum) [3][C][threads] and the replicate's shift [threads] --
    // shared memory, so registers hold the march's own working set
    extern __shared__ float4 s_dyn[];
    const int nthr = blockDim.x;
    float2 *const slk = reinterpret_cast<float2 *>(s_dyn) + (threadIdx.x >> 5) * P.slab_len;
    const float2 *const sli = slk + P.slab_klen;
    double *const s_acc = reinterpret_cast<double *>(reinterpret_cast<float2 *>(s_dyn) + ((nthr + 31) >> 5) * P.slab_len);
    uint4 *const s_shift = reinterpret_cast<uint4 *>(s_acc + 3 * C * nthr);
    auto acc = [&](int q, int k) { return s_acc + (q * C + k) * nthr + tid; };
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
        const bool act_a = a0 < P.ea1;
        const int acl = act_a ? a0 : P.ea0;  // cells outside the region march a valid cell, untallied
        bool active[C];
        int bcl[C], tcell[C];
#pragma unroll
        for (int k = 0; k < C; ++k) {
            const int b0 = P.eb0 + pb * P.tile_b + lb + k * hb;
            active[k] = act_a && b0 < P.eb1;
            bcl[k] = active[k] ? b0 : P.eb0;
            tcell[k] = ((w0 - P.ew0) * nkR + (bcl[k] - P.eb0)) * njR + (acl - P.ea0);
        }
        const int N = P.rays_per_packet ? P.rays_per_packet[G * P.rays_gstride + p] : P.rays;
        const long long fbase = (long long)f * P.field_stride;
        const int rowW0 = w0 * plane;
        const float oW = (__ldg(P.fw + w0) + __ldg(P.fw + w0 + 1)) * 0.5f;
        // alias table of this packet: band group G of the temperature bin
        // nearest to the temperature of the packet's first cell
        int gs = 0, K = 1;
        if constexpr (MODE == MODE_GREY) {
#pragma unroll
            for (int k = 0; k < C; ++k) {
                const float Ti = load_field<MODE>(P, fbase, rowW0 + bcl[k] * P.na + acl);
                if (!(Ti > 0.0f) && active[k]) flags |= DNSMC_STATUS_BAD_FIELD;
            }
        } else {
            int boff = 0;
            if (P.n_tbins > 1) {
                int kx, ti;
                float ft, fx;
                cell_coords<MODE>(load_field<MODE>(P, fbase, rowW0 + bcl[0] * P.na + acl), &kx, &ti, &ft, &fx);
                const float tp0 = __shfl_sync(FULL, (float)ti + ft, 0);
                int bin = __float2int_rn(tp0);
                bin = min(max(bin, 0), P.n_tbins - 1);
                boff = bin * P.n_groups;
            }
            gs = P.group_start[boff + G];
            K = P.group_start[boff + G + 1] - gs;
        }
        const uint32_t ctr2 = (uint32_t)G | ((uint32_t)(f + P.field_base) << 16);
        double mo[C][9];
        if (MOM)
#pragma unroll
            for (int k = 0; k < C; ++k)
#pragma unroll
                for (int q = 0; q < 9; ++q) mo[k][q] = 0.0;
        const int M = P.sampler ? max(1, N / max(1, P.nbatch)) : 1;
#pragma unroll
        for (int k = 0; k < C; ++k) { *acc(0, k) = 0.0; *acc(1, k) = 0.0; *acc(2, k) = 0.0; }
        unsigned long long isteps = 0;
        unsigned int lsteps = 0;  // this lane's active cell-steps in the item
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

            // spectral sample, each cell's own k, Ib and weight wk
            int nbnd = 0, sid = 0;
            float wk[C], Ii[C];
            VT vcur[C];
#pragma unroll
            for (int k = 0; k < C; ++k) vcur[k] = load_field<MODE>(P, fbase, rowW0 + bcl[k] * P.na + acl);
            if constexpr (MODE == MODE_GREY) {
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    const float Ti = vcur[k];
                    const float t2 = Ti * Ti;
                    Ii[k] = t2 * t2;
                    wk[k] = P.Wgrey;
                }
            } else {
                const int j = (int)__umulhi(x.z, (uint32_t)K);
                SpecEntry e = P.entries[gs + j];
                if (!(u24(x.w) < e.prob)) e = P.entries[gs + (int)(e.alias_nb & 0xFFFFu)];
                nbnd = (int)(e.alias_nb >> 16);
                sid = e.koff;
                if (!load_slab(P, sid, slk, lane, sbar, &sphase, &flags)) { dead = true; break; }
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    int kx, ti;
                    float ft, fx;
                    cell_coords<MODE>(vcur[k], &kx, &ti, &ft, &fx);
                    const float ki = lookup_k<MODE>(slk, kx, ft, fx);
                    Ii[k] = lookup_ib(sli, ti, ft);
                    wk[k] = e.W * ki;
                }
            }

            // warp-uniform DDA from the cell centres
            const float invW = 1.0f / fabsf(sW), invA = 1.0f / fabsf(sA), invB = 1.0f / fabsf(sB);
            const int dW = sW > 0.f ? 1 : -1, dA = sA > 0.f ? 1 : -1, dB = sB > 0.f ? 1 : -1;
            // crossing parameter of the next wall-normal face: (fw[c + 1] - o) / s
            // going up, (o - fw[c]) / |s| = (fw[c] - o) * (-1/|s|) going down
            // (negation is exact: the same values)
            const float *fwn = P.fw + (dW > 0 ? 1 : 0);
            const float sinvW = dW > 0 ? invW : -invW;
            float tW = (__ldg(fwn + w0) - oW) * sinvW;
            // periodic wrap of the next j / k index: one compare per step
            const int wrapA = dA > 0 ? P.na : -1, resetA = dA > 0 ? 0 : P.na - 1;
            // k moves as its row offset k * na: one step is +-na, the wrap
            // compares against the offset one row past the end
            const int dRowB = dB * P.na;
            const int wrapRowB = dB > 0 ? P.nb * P.na : -P.na, resetRowB = dB > 0 ? 0 : (P.nb - 1) * P.na;
            const int wallW = dW > 0 ? P.nw : -1;  // the wall-normal index beyond the wall
            const int dRowW = dW * plane;
            const float dtA = P.da * invA, dtB = P.db * invB;
            float tA = 0.5f * dtA, tB = 0.5f * dtB;
            // crossing counts plus one half, as floats: (float)n + 0.5f is
            // exact and so is adding 1 to it below 2^22 crossings, so these
            // are the values the integer counts would give, without a
            // conversion per step
            float hA = 0.5f, hB = 0.5f;
            int cw = w0, ca = acl, rowW = rowW0;
            int rowB[C];
            float tau[C], D[C];
#pragma unroll
            for (int k = 0; k < C; ++k) {
                rowB[k] = bcl[k] * P.na;
                tau[k] = active[k] ? 1.0f : 0.0f;
                D[k] = 0.0f;
            }
            float t = 0.0f;
            int steps = 0;
            // the step at which each cell was dumped (its live steps are that
            // plus one; cells never dumped were live for every step)
            int life[C];
#pragma unroll
            for (int k = 0; k < C; ++k) life[k] = 1 << 30;
            // two steps per pass, each its own copy of the body (the current /
            // next field values alternate registers instead of being copied),
            // the warp's exit vote after the second
            for (;;) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const bool sW_ = tW <= tA && tW <= tB;
                    const bool sA_ = !sW_ && tA <= tB;
                    const int axis = sW_ ? 0 : (sA_ ? 1 : 2);
                    const float tn = sW_ ? tW : (sA_ ? tA : tB);
                    const float ds = tn - t;
                    const float nds = t - tn;  // minus the segment length (exact negation)
                    // next cell of the walk, and its field values fetched now; the
                    // axis is the same in every lane, but selects cost fewer
                    // instructions here than branches the compiler must treat as
                    // divergent
                    int ncw, nca, nrowW;
                    int nrowB[C];
                    const bool aW = axis == 0, aA = axis == 1, aB = axis == 2;
                    ncw = aW ? cw + dW : cw;
                    nrowW = aW ? rowW + dRowW : rowW;
                    {
                        int u = ca + dA;
                        u = u == wrapA ? resetA : u;
                        nca = aA ? u : ca;
                    }
#pragma unroll
                    for (int k = 0; k < C; ++k) {
                        int u = rowB[k] + dRowB;
                        u = u == wrapRowB ? resetRowB : u;
                        nrowB[k] = aB ? u : rowB[k];
                    }
                    const bool wall = aW && ncw == wallW;
                    // fetched for every cell, live or not (a dumped cell's value
                    // is never used): no default copy, no per-cell predicate; at
                    // a wall the row stays inside the grid and the walk ends
                    const int lrowW = wall ? rowW : nrowW;
                    VT vnext[C];
#pragma unroll
                    for (int k = 0; k < C; ++k) vnext[k] = load_field<MODE>(P, fbase, lrowW + nrowB[k] + nca);
                    // attenuation and collected intensity of this segment; a cell
                    // already dumped (tau 0) adds exactly nothing.  Per cell:
                    // alpha = -expm1(-k ds), ta = tau alpha, D += ta g,
                    // tau -= ta, with g = Ii - Ib_j: D is the net exchange in
                    // intensity units and the ray's contribution wk D (the
                    // reference normalises g by Ii and multiplies the ray by Ii
                    // again; without the two the march saves a multiply per
                    // cell-step and a division per ray, and a cell whose Ii
                    // underflows keeps its absorption).  The two cells of a
                    // pair go through paired FP32 instructions with every sign
                    // moved onto an operand whose negation is exact: e =
                    // expm1(k * (t - tn)) = -alpha, nta = tau e = -ta,
                    // D += nta (-g), tau += nta -- the same roundings.
                    bool dumped[C];  // after this step: tau 0 (dumped now or before)
#pragma unroll
                    for (int k = 0; k < C; k += 2) {
                        float kj[2], ngj[2];
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            if constexpr (MODE == MODE_GREY) {
                                const float t2 = vcur[k + h] * vcur[k + h];
                                ngj[h] = t2 * t2 - Ii[k + h];
                                kj[h] = P.kappa;
                            } else {
                                int kx, tj;
                                float ftj, fxj;
                                cell_coords<MODE>(vcur[k + h], &kx, &tj, &ftj, &fxj);
                                kj[h] = lookup_k<MODE>(slk, kx, ftj, fxj);
                                const float Ibj = lookup_ib(sli, tj, ftj);
                                ngj[h] = Ibj - Ii[k + h];
                            }
                        }
                        const float2 e = mc_expm1_x2(__fmul2_rn(make_float2(kj[0], kj[1]), make_float2(nds, nds)));
                        const float2 nta = __fmul2_rn(make_float2(tau[k], tau[k + 1]), e);
                        const float2 d2 = __ffma2_rn(nta, make_float2(ngj[0], ngj[1]), make_float2(D[k], D[k + 1]));
                        const float2 t2 = __fadd2_rn(make_float2(tau[k], tau[k + 1]), nta);
                        D[k] = d2.x; D[k + 1] = d2.y;
                        tau[k] = t2.x; tau[k + 1] = t2.y;
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            dumped[k + h] = tau[k + h] < P.toll;
                            if (dumped[k + h]) {
                                D[k + h] = fmaf(-tau[k + h], ngj[h], D[k + h]);
                                tau[k + h] = 0.0f;
                                life[k + h] = min(life[k + h], steps);
                            }
                        }
                    }
                    if (TRACE && lane == 0 && steps < P.trace_max) {
                        int *rec = P.trace_rec + 6 * steps;
                        rec[0] = cw; rec[1] = dA * (int)(hA - 0.5f); rec[2] = dB * (int)(hB - 0.5f); rec[3] = axis;
                        rec[4] = __float_as_int(ds); rec[5] = __float_as_int(tau[0]);
                    }
                    t = tn;
                    ++steps;
                    {
                        if (wall) {
                            const int side = ncw < 0 ? 0 : 1;
                            const float Iw = (MODE == MODE_GREY) ? P.Tw4[side] : __ldg(P.ibw + side * P.nbands + nbnd);
#pragma unroll
                            for (int k = 0; k < C; ++k) {
                                D[k] = fmaf(tau[k], Ii[k] - Iw, D[k]);
                                tau[k] = 0.0f;
                            }
                            goto walk_end;
                        }
                        cw = ncw;
                        rowW = nrowW;
                        if (aW) tW = (__ldg(fwn + cw) - oW) * sinvW;
                        hA = aA ? hA + 1.0f : hA;
                        tA = hA * dtA;
                        ca = nca;
                        hB = aB ? hB + 1.0f : hB;
                        tB = hB * dtB;
#pragma unroll
                        for (int k = 0; k < C; ++k) rowB[k] = nrowB[k];
                    }
#pragma unroll
                    for (int k = 0; k < C; ++k) vcur[k] = vnext[k];
                    // a cell not dumped has tau >= toll > 0
                    bool alive = false;
#pragma unroll
                    for (int k = 0; k < C; ++k) alive = alive || !dumped[k];
                    if (steps >= P.max_steps) {
                        if (alive) flags |= DNSMC_STATUS_STEP_CAP;
                        goto walk_end;
                    }
                    if (u == 1 && !__any_sync(FULL, alive)) goto walk_end;
                }
            }
        walk_end:
            {
                // the exit vote comes every second step, so a walk may take
                // one step past the one that dumped the warp's last live
                // cell; that step changes nothing (every tau is 0 and the
                // cells stay in the grid), and the walk's length is the last
                // dump step plus one (never dumped: 2^30, no change)
                int last = 0;
#pragma unroll
                for (int k = 0; k < C; ++k) last = max(last, life[k]);
                last = __reduce_max_sync(FULL, last);
                steps = min(steps, last + 1);
            }
            if (TRACE && lane == 0) *P.trace_n = steps;
#pragma unroll
            for (int k = 0; k < C; ++k) lsteps += active[k] ? (unsigned)min(life[k] + 1, steps) : 0u;
            isteps += (unsigned long long)steps;
            // control variate: the ray's straight flight through the
            // layer-mean medium, the same for both cells (same layer)
            float Jbar = 0.0f, Aown = 0.0f, I0 = 0.0f;
            if (CV) {
                const long long srow = ((long long)f * P.n_samples + sid) * P.nw + w0;
                I0 = __ldg(P.sur + srow).y;
                surrogate_lookup(P.surtab + srow * (2 * kSurBins), sW, &Jbar, &Aown);
            }
#pragma unroll
            for (int k = 0; k < C; ++k) {
                float X = wk[k] * D[k];
                if (CV) {
                    // Y_a: the ray through the layer-mean medium; Y_b: its own-layer part
                    const float Ya = wk[k] * (Ii[k] - Jbar);
                    const float Yb = wk[k] * (Aown * (Ii[k] - I0));
                    if (MOM && active[k]) {
                        const double xd = X, ya = Ya, yb = Yb;
                        mo[k][0] += xd; mo[k][1] += ya; mo[k][2] += yb;
                        mo[k][3] = fma(xd, xd, mo[k][3]); mo[k][4] = fma(ya, ya, mo[k][4]);
                        mo[k][5] = fma(yb, yb, mo[k][5]); mo[k][6] = fma(xd, ya, mo[k][6]);
                        mo[k][7] = fma(xd, yb, mo[k][7]); mo[k][8] = fma(ya, yb, mo[k][8]);
                    }
                    const float2 beta = P.beta ? P.beta[fg * P.region_cells + tcell[k]] : make_float2(1.0f, -1.0f);
                    X = X - beta.x * Ya;  // tallied: X - beta_a Y_a - beta_b Y_b; the
                    X = X - beta.y * Yb;  // means beta . E[Y] are added back at finalize
                }
                if (active[k]) {
                    ++my_rays;
                    if (!isfinite(X)) flags |= DNSMC_STATUS_NONFINITE;
                    tally_ray(P, X, m, M, reinterpret_cast<float2 *>(acc(0, k)), reinterpret_cast<float2 *>(acc(1, k)),
                              reinterpret_cast<float2 *>(acc(2, k)));
                }
            }
        }
        if (dead) break;  // the item's sums are incomplete; the solve fails
        my_steps += lsteps;
        if (TRACE) return;
        if (P.item_steps && lane == 0) P.item_steps[item] = isteps;
#pragma unroll
        for (int k = 0; k < C; ++k) {
            if (!active[k]) continue;
            const long long o = fg * P.region_cells + tcell[k];
            P.tally[o] = make_double2(ff_value(*reinterpret_cast<const float2 *>(acc(0, k))),
                                      ff_value(*reinterpret_cast<const float2 *>(acc(1, k))));
            if (MOM) {
                double *out = P.moments + o * 9;
#pragma unroll
                for (int q = 0; q < 9; ++q) out[q] = mo[k][q];
            }
        }
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

// ---------------------------------------------------------------------------
// The same march for the general medium (GEN): particles with scattering and
// grey diffuse walls; restarts of the walk at every scattering and wall
// reflection, so the crossing counts are integers with the restart offsets.
// ---------------------------------------------------------------------------
template <int MODE, bool TRACE, bool CV, bool MOM>
__global__ void __launch_bounds__(256, DNSMC_PAIR_MINB) march_gen_kernel(const MarchParams P) {
    typedef typename FieldT<MODE>::type VT;
    const float INF = __int_as_float(0x7f800000);
    constexpr int C = kLaneCells;  // cells per lane
    static_assert(C % 2 == 0, "the attenuation goes through cell pairs");
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int tid = threadIdx.x;
    const int la = lane % P.tile_a, lb = lane / P.tile_a;
    const int hb = 32 / P.tile_a;  // k rows between a lane's two cells
    const int njR = P.ea1 - P.ea0, nkR = P.eb1 - P.eb0;
    const int plane = P.na * P.nb;
    unsigned long long my_rays = 0, my_steps = 0;
    unsigned int flags = 0;
    // dynamic shared memory (march_smem): this warp's copy of the current
    // ray's table slab (tabulated models); per-cell sums of the item as
    // float pairs (ray sum, sum of squares or of squared replicate means,
    // current replicate sum) [3][C][threads] and the replicate's shift [threads] --
    // shared memory, so registers hold the march's own working set
    extern __shared__ float4 s_dyn[];
    const int nthr = blockDim.x;
    float2 *const slk = reinterpret_cast<float2 *>(s_dyn) + (threadIdx.x >> 5) * P.slab_len;
    const float2 *const sli = slk + P.slab_klen;
    double *const s_acc = reinterpret_cast<double *>(reinterpret_cast<float2 *>(s_dyn) + ((nthr + 31) >> 5) * P.slab_len);
    uint4 *const s_shift = reinterpret_cast<uint4 *>(s_acc + 3 * C * nthr);
    auto acc = [&](int q, int k) { return s_acc + (q * C + k) * nthr + tid; };
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
        const bool act_a = a0 < P.ea1;
        const int acl = act_a ? a0 : P.ea0;  // cells outside the region march a valid cell, untallied
        bool active[C];
        int bcl[C], tcell[C];
#pragma unroll
        for (int k = 0; k < C; ++k) {
            const int b0 = P.eb0 + pb * P.tile_b + lb + k * hb;
            active[k] = act_a && b0 < P.eb1;
            bcl[k] = active[k] ? b0 : P.eb0;
            tcell[k] = ((w0 - P.ew0) * nkR + (bcl[k] - P.eb0)) * njR + (acl - P.ea0);
        }
        const int N = P.rays_per_packet ? P.rays_per_packet[G * P.rays_gstride + p] : P.rays;
        const long long fbase = (long long)f * P.field_stride;
        const int rowW0 = w0 * plane;
        const float oW = (__ldg(P.fw + w0) + __ldg(P.fw + w0 + 1)) * 0.5f;
        // alias table of this packet: band group G of the temperature bin
        // nearest to the temperature of the packet's first cell
        int gs = 0, K = 1;
        if constexpr (MODE == MODE_GREY) {
#pragma unroll
            for (int k = 0; k < C; ++k) {
                const float Ti = load_field<MODE>(P, fbase, rowW0 + bcl[k] * P.na + acl);
                if (!(Ti > 0.0f) && active[k]) flags |= DNSMC_STATUS_BAD_FIELD;
            }
        } else {
            int boff = 0;
            if (P.n_tbins > 1) {
                int kx, ti;
                float ft, fx;
                cell_coords<MODE>(load_field<MODE>(P, fbase, rowW0 + bcl[0] * P.na + acl), &kx, &ti, &ft, &fx);
                const float tp0 = __shfl_sync(FULL, (float)ti + ft, 0);
                int bin = __float2int_rn(tp0);
                bin = min(max(bin, 0), P.n_tbins - 1);
                boff = bin * P.n_groups;
            }
            gs = P.group_start[boff + G];
            K = P.group_start[boff + G + 1] - gs;
        }
        const uint32_t ctr2 = (uint32_t)G | ((uint32_t)(f + P.field_base) << 16);
        double mo[C][9];
        if (MOM)
#pragma unroll
            for (int k = 0; k < C; ++k)
#pragma unroll
                for (int q = 0; q < 9; ++q) mo[k][q] = 0.0;
        const int M = P.sampler ? max(1, N / max(1, P.nbatch)) : 1;
#pragma unroll
        for (int k = 0; k < C; ++k) { *acc(0, k) = 0.0; *acc(1, k) = 0.0; *acc(2, k) = 0.0; }
        unsigned long long isteps = 0;
        unsigned int lsteps = 0;  // this lane's active cell-steps in the item
        int bcur = -1;
        const int rbeg = TRACE ? P.trace_r : 0;
        const int rend = TRACE ? P.trace_r + 1 : ((K > 0) ? N : 0);
        for (int r = rbeg; r < rend; ++r) {
            int m;
            const uint4 x = ray_words(P, r, M, p, ctr2, &bcur, &s_shift[tid], &m);
            if (TRACE && lane == 0) {
                P.trace_rng[0] = x.x; P.trace_rng[1] = x.y; P.trace_rng[2] = x.z; P.trace_rng[3] = x.w;
            }
            float sW_e, sA_e, sB_e;  // the emission direction
            ray_direction(x, &sW_e, &sA_e, &sB_e);

            // spectral sample, each cell's own k, Ib and weight wk
            int nbnd = 0, sid = 0;
            float wk[C], Ii[C];
            VT vcur[C];
            float fvcur[C];  // the particle volume fraction of the current cells
            float pab = 0.0f, psc = 0.0f;  // particle absorption / scattering per unit volume fraction
#pragma unroll
            for (int k = 0; k < C; ++k) {
                vcur[k] = load_field<MODE>(P, fbase, rowW0 + bcl[k] * P.na + acl);
                fvcur[k] = P.fieldV ? __ldg(P.fieldV + fbase + rowW0 + bcl[k] * P.na + acl) : 0.0f;
            }
            if constexpr (MODE == MODE_GREY) {
                if (P.part) { const float2 pp = __ldg(P.part); pab = pp.x; psc = pp.y; }
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    const float Ti = vcur[k];
                    const float t2 = Ti * Ti;
                    Ii[k] = t2 * t2;
                    wk[k] = P.W4sig * fmaf(fvcur[k], pab, P.kappa);
                }
            } else {
                const int j = (int)__umulhi(x.z, (uint32_t)K);
                SpecEntry e = P.entries[gs + j];
                if (!(u24(x.w) < e.prob)) e = P.entries[gs + (int)(e.alias_nb & 0xFFFFu)];
                nbnd = (int)(e.alias_nb >> 16);
                sid = e.koff;
                if (!load_slab(P, sid, slk, lane, sbar, &sphase, &flags)) { dead = true; break; }
                if (P.part) { const float2 pp = __ldg(P.part + nbnd); pab = pp.x; psc = pp.y; }
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    int kx, ti;
                    float ft, fx;
                    cell_coords<MODE>(vcur[k], &kx, &ti, &ft, &fx);
                    float ki = lookup_k<MODE>(slk, kx, ft, fx);
                    ki = fmaf(fvcur[k], pab, ki);
                    Ii[k] = lookup_ib(sli, ti, ft);
                    wk[k] = e.W * ki;
                }
            }

            // warp-uniform DDA from (pw0, fa0, fb0): the wall-normal coordinate
            // and the fractional offsets inside the current periodic cells (the
            // cell centres at emission, restarted at every scattering and wall
            // reflection)
            float sW = sW_e, sA = sA_e, sB = sB_e;
            float pw0 = oW, fa0 = 0.5f, fb0 = 0.5f, offA = 0.5f, offB = 0.5f;
            float invW, invA, invB, sinvW, tW, dtA, dtB, tA, tB;
            int dW, dA, dB, nA = 0, nB = 0;
            // per direction: the exit face (fw[c + 1] - o)/s going up, (fw[c] - o)
            // * (-1/|s|) going down (the values of (o - fw[c])/|s|: negation is
            // exact), the index beyond the wall, the one-compare periodic wraps
            const float *fwn;
            int wallW, dRowW, wrapA, resetA, wrapB, resetB;
            int cw = w0;
            auto dda_init = [&]() {
                invW = 1.0f / fabsf(sW); invA = 1.0f / fabsf(sA); invB = 1.0f / fabsf(sB);
                dW = sW > 0.f ? 1 : -1; dA = sA > 0.f ? 1 : -1; dB = sB > 0.f ? 1 : -1;
                fwn = P.fw + (dW > 0 ? 1 : 0);
                sinvW = dW > 0 ? invW : -invW;
                wallW = dW > 0 ? P.nw : -1;
                dRowW = dW * plane;
                wrapA = dA > 0 ? P.na : -1; resetA = dA > 0 ? 0 : P.na - 1;
                wrapB = dB > 0 ? P.nb : -1; resetB = dB > 0 ? 0 : P.nb - 1;
                tW = (__ldg(fwn + cw) - pw0) * sinvW;
                dtA = P.da * invA; dtB = P.db * invB;
                offA = dA > 0 ? 1.0f - fa0 : fa0;
                offB = dB > 0 ? 1.0f - fb0 : fb0;
                tA = offA * dtA; tB = offB * dtB;
                nA = 0; nB = 0;
            };
            dda_init();
            int ca = acl, rowW = rowW0;
            int cb[C], rowB[C];
            float tau[C], D[C];
#pragma unroll
            for (int k = 0; k < C; ++k) {
                cb[k] = bcl[k];
                rowB[k] = bcl[k] * P.na;
                tau[k] = active[k] ? 1.0f : 0.0f;
                D[k] = 0.0f;
            }
            float t = 0.0f;
            int steps = 0;
            // scattering events: one Philox word quadruple per event
            uint32_t ev = 0;
            uint4 evx = make_uint4(0u, 0u, 0u, 0u);
            float sigbar = 0.0f, tcol = INF;
            auto draw = [&]() {
                evx = philox4x32_10(make_uint4((uint32_t)r, (uint32_t)p, ctr2, 0x5CA70000u + ev), P.key0, P.key1);
                ++ev;
            };
            sigbar = P.fv_max * psc;
            if (sigbar > 0.0f) { draw(); tcol = mc_neglog(u24o(evx.x)) / sigbar; }
            // unrolled by two: the current / next field values alternate
            // registers instead of being copied every step
#pragma unroll 2
            for (;;) {
                const bool sW_ = tW <= tA && tW <= tB;
                const bool sA_ = !sW_ && tA <= tB;
                int axis = sW_ ? 0 : (sA_ ? 1 : 2);
                float tn = sW_ ? tW : (sA_ ? tA : tB);
                {  // a tentative collision first
                    const bool col = tcol < tn;
                    axis = col ? 3 : axis;
                    tn = col ? tcol : tn;
                }
                const float ds = tn - t;
                const float nds = t - tn;  // minus the segment length (exact negation)
                // next cell of the walk, and its field values fetched now; the
                // axis is the same in every lane, but selects cost fewer
                // instructions here than branches the compiler must treat as
                // divergent
                int ncw, nca, nrowW;
                int ncb[C], nrowB[C];
                const bool aW = axis == 0, aA = axis == 1, aB = axis == 2;
                ncw = aW ? cw + dW : cw;
                nrowW = aW ? rowW + dRowW : rowW;
                {
                    int u = ca + dA;
                    u = u == wrapA ? resetA : u;
                    nca = aA ? u : ca;
                }
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    int u = cb[k] + dB;
                    u = u == wrapB ? resetB : u;
                    ncb[k] = aB ? u : cb[k];
                    nrowB[k] = aB ? u * P.na : rowB[k];
                }
                const bool wall = aW && ncw == wallW;
                // fetched for every cell, live or not (a dumped cell's value
                // is never used); a collision keeps the cell, so the address
                // is the current one, and at a wall the row stays inside the
                // grid and the walk restarts or ends
                const int lrowW = wall ? rowW : nrowW;
                VT vnext[C];
                float fvnext[C];
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    vnext[k] = load_field<MODE>(P, fbase, lrowW + nrowB[k] + nca);
                    fvnext[k] = P.fieldV ? __ldg(P.fieldV + fbase + lrowW + nrowB[k] + nca) : fvcur[k];
                }
                // attenuation and collected intensity of this segment; a cell
                // already dumped (tau 0) adds exactly nothing.  The same
                // paired update as the gas march: e = expm1(k * (t - tn)) =
                // -alpha, nta = tau e = -ta, D += nta (-g), tau += nta.
#pragma unroll
                for (int k = 0; k < C; k += 2) {
                    float kj[2], ngj[2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        lsteps += tau[k + h] > 0.0f ? 1u : 0u;
                        if constexpr (MODE == MODE_GREY) {
                            const float t2 = vcur[k + h] * vcur[k + h];
                            ngj[h] = t2 * t2 - Ii[k + h];
                            kj[h] = P.kappa;
                        } else {
                            int kx, tj;
                            float ftj, fxj;
                            cell_coords<MODE>(vcur[k + h], &kx, &tj, &ftj, &fxj);
                            kj[h] = lookup_k<MODE>(slk, kx, ftj, fxj);
                            const float Ibj = lookup_ib(sli, tj, ftj);
                            ngj[h] = Ibj - Ii[k + h];
                        }
                        kj[h] = fmaf(fvcur[k + h], pab, kj[h]);
                    }
                    const float2 e = mc_expm1_x2(__fmul2_rn(make_float2(kj[0], kj[1]), make_float2(nds, nds)));
                    const float2 nta = __fmul2_rn(make_float2(tau[k], tau[k + 1]), e);
                    const float2 d2 = __ffma2_rn(nta, make_float2(ngj[0], ngj[1]), make_float2(D[k], D[k + 1]));
                    const float2 t2 = __fadd2_rn(make_float2(tau[k], tau[k + 1]), nta);
                    D[k] = d2.x; D[k + 1] = d2.y;
                    tau[k] = t2.x; tau[k + 1] = t2.y;
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        if (tau[k + h] < P.toll) { D[k + h] = fmaf(-tau[k + h], ngj[h], D[k + h]); tau[k + h] = 0.0f; }
                }
                if (TRACE && lane == 0 && steps < P.trace_max) {
                    int *rec = P.trace_rec + 6 * steps;
                    rec[0] = cw; rec[1] = dA * nA; rec[2] = dB * nB; rec[3] = axis;
                    rec[4] = __float_as_int(ds); rec[5] = __float_as_int(tau[0]);
                }
                t = tn;
                ++steps;
                {
                    if (wall) {
                        const int side = ncw < 0 ? 0 : 1;
                        const float Iw = (MODE == MODE_GREY) ? P.Tw4[side] : __ldg(P.ibw + side * P.nbands + nbnd);
                        {
                            // grey wall: it takes eps of the throughput at its
                            // own intensity and reflects the rest diffusely
                            const float eps = P.eps[side];
                            bool live = false;
#pragma unroll
                            for (int k = 0; k < C; ++k) {
                                if (tau[k] > 0.0f) {
                                    const float gw = Ii[k] - Iw;
                                    D[k] = fmaf(tau[k] * eps, gw, D[k]);
                                    tau[k] = eps >= 1.0f ? 0.0f : tau[k] * (1.0f - eps);
                                    if (tau[k] > 0.0f && tau[k] < P.toll) { D[k] = fmaf(tau[k], gw, D[k]); tau[k] = 0.0f; }
                                }
                                live = live || tau[k] > 0.0f;
                            }
                            if (!__any_sync(FULL, live)) break;
                            // diffuse reflection from the wall point
                            const float ta_ = t / dtA, tb_ = t / dtB;
                            fa0 = dA > 0 ? fa0 + (ta_ - (float)nA) : fa0 - (ta_ - (float)nA);
                            fb0 = dB > 0 ? fb0 + (tb_ - (float)nB) : fb0 - (tb_ - (float)nB);
                            fa0 = fminf(fmaxf(fa0, 0.0f), 1.0f);
                            fb0 = fminf(fmaxf(fb0, 0.0f), 1.0f);
                            pw0 = side == 0 ? __ldg(P.fw) : __ldg(P.fw + P.nw);
                            draw();  // this event's words: the reflected direction only
                            const float cmu = sqrtf(u24(evx.z));
                            const float smu = sqrtf(fmaxf(0.0f, 1.0f - cmu * cmu));
                            float cp, sp;
                            mc_sincos_turn(evx.w >> 8, &cp, &sp);
                            sW = side == 0 ? cmu : -cmu;
                            sA = smu * cp;
                            sB = smu * sp;
                            dda_init();
                            t = 0.0f;
                            if (sigbar > 0.0f) { draw(); tcol = mc_neglog(u24o(evx.x)) / sigbar; }
                            if (steps >= P.max_steps) {
                                if (live) flags |= DNSMC_STATUS_STEP_CAP;
                                break;
                            }
                            continue;
                        }
                    }
                    cw = ncw;
                    rowW = nrowW;
                    if (aW) tW = (__ldg(fwn + cw) - pw0) * sinvW;
                    ca = nca;
#pragma unroll
                    for (int k = 0; k < C; ++k) { cb[k] = ncb[k]; rowB[k] = nrowB[k]; }
                    nA += aA ? 1 : 0;
                    tA = aA ? ((float)nA + offA) * dtA : tA;
                    nB += aB ? 1 : 0;
                    tB = aB ? ((float)nB + offB) * dtB : tB;
                }
                if (axis == 3) {
                    // tentative collision: shared decision, per-cell weights
                    float pl[C];
                    float ps = 0.0f, pc = 0.0f;
#pragma unroll
                    for (int k = 0; k < C; ++k) {
                        pl[k] = tau[k] > 0.0f ? fminf(1.0f, fvcur[k] * psc / sigbar) : 0.0f;
                        ps = k == 0 ? pl[k] : ps + pl[k];
                        pc = k == 0 ? (tau[k] > 0.0f ? 1.0f : 0.0f) : pc + (tau[k] > 0.0f ? 1.0f : 0.0f);
                    }
                    for (int o = 16; o > 0; o >>= 1) {
                        ps += __shfl_xor_sync(FULL, ps, o);
                        pc += __shfl_xor_sync(FULL, pc, o);
                    }
                    const float q = pc > 0.0f ? ps / pc : 0.0f;
                    if (u24(evx.y) < q) {
#pragma unroll
                        for (int k = 0; k < C; ++k)
                            if (tau[k] > 0.0f) tau[k] = tau[k] * (pl[k] / q);
                        const float ta_ = t / dtA, tb_ = t / dtB;
                        fa0 = dA > 0 ? fa0 + (ta_ - (float)nA) : fa0 - (ta_ - (float)nA);
                        fb0 = dB > 0 ? fb0 + (tb_ - (float)nB) : fb0 - (tb_ - (float)nB);
                        fa0 = fminf(fmaxf(fa0, 0.0f), 1.0f);
                        fb0 = fminf(fmaxf(fb0, 0.0f), 1.0f);
                        pw0 = fminf(fmaxf(fmaf(sW, t, pw0), __ldg(P.fw + cw)), __ldg(P.fw + cw + 1));
                        hg_scatter(P.hg_g, evx.z, evx.w, &sW, &sA, &sB);
                        dda_init();
                        t = 0.0f;
                    } else {
#pragma unroll
                        for (int k = 0; k < C; ++k)
                            if (tau[k] > 0.0f) tau[k] = tau[k] * ((1.0f - pl[k]) / (1.0f - q));
                    }
                    draw();
                    tcol = t + mc_neglog(u24o(evx.x)) / sigbar;
                }
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    vcur[k] = vnext[k];
                    fvcur[k] = fvnext[k];
                }
                bool alive = false;
#pragma unroll
                for (int k = 0; k < C; ++k) alive = alive || tau[k] > 0.0f;
                if (!__any_sync(FULL, alive)) break;
                if (steps >= P.max_steps) {
                    if (alive) flags |= DNSMC_STATUS_STEP_CAP;
                    break;
                }
            }
            if (TRACE && lane == 0) *P.trace_n = steps;
            isteps += (unsigned long long)steps;
            // control variate: the ray's straight flight through the
            // layer-mean medium, the same for both cells (same layer)
            float Jbar = 0.0f, Aown = 0.0f, I0 = 0.0f;
            if (CV) {
                const long long srow = ((long long)f * P.n_samples + sid) * P.nw + w0;
                I0 = __ldg(P.sur + srow).y;
                surrogate_lookup(P.surtab + srow * (2 * kSurBins), sW_e, &Jbar, &Aown);
            }
#pragma unroll
            for (int k = 0; k < C; ++k) {
                float X = wk[k] * D[k];
                if (CV) {
                    // Y_a: the ray through the layer-mean medium; Y_b: its own-layer part
                    const float Ya = wk[k] * (Ii[k] - Jbar);
                    const float Yb = wk[k] * (Aown * (Ii[k] - I0));
                    if (MOM && active[k]) {
                        const double xd = X, ya = Ya, yb = Yb;
                        mo[k][0] += xd; mo[k][1] += ya; mo[k][2] += yb;
                        mo[k][3] = fma(xd, xd, mo[k][3]); mo[k][4] = fma(ya, ya, mo[k][4]);
                        mo[k][5] = fma(yb, yb, mo[k][5]); mo[k][6] = fma(xd, ya, mo[k][6]);
                        mo[k][7] = fma(xd, yb, mo[k][7]); mo[k][8] = fma(ya, yb, mo[k][8]);
                    }
                    const float2 beta = P.beta ? P.beta[fg * P.region_cells + tcell[k]] : make_float2(1.0f, -1.0f);
                    X = X - beta.x * Ya;  // tallied: X - beta_a Y_a - beta_b Y_b; the
                    X = X - beta.y * Yb;  // means beta . E[Y] are added back at finalize
                }
                if (active[k]) {
                    ++my_rays;
                    if (!isfinite(X)) flags |= DNSMC_STATUS_NONFINITE;
                    tally_ray(P, X, m, M, reinterpret_cast<float2 *>(acc(0, k)), reinterpret_cast<float2 *>(acc(1, k)),
                              reinterpret_cast<float2 *>(acc(2, k)));
                }
            }
        }
        if (dead) break;  // the item's sums are incomplete; the solve fails
        my_steps += lsteps;
        if (TRACE) return;
        if (P.item_steps && lane == 0) P.item_steps[item] = isteps;
#pragma unroll
        for (int k = 0; k < C; ++k) {
            if (!active[k]) continue;
            const long long o = fg * P.region_cells + tcell[k];
            P.tally[o] = make_double2(ff_value(*reinterpret_cast<const float2 *>(acc(0, k))),
                                      ff_value(*reinterpret_cast<const float2 *>(acc(1, k))));
            if (MOM) {
                double *out = P.moments + o * 9;
#pragma unroll
                for (int q = 0; q < 9; ++q) out[q] = mo[k][q];
            }
        }
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

// The two-cell march of a medium: the absorbing gas (march_pair_kernel) or
// the general medium (march_gen_kernel).
template <int MODE, bool TRACE, bool CV, bool MOM, bool GEN> struct march_cells_kernel {
    static constexpr void (*fn)(const MarchParams) = march_pair_kernel<MODE, TRACE, CV, MOM>;
};
template <int MODE, bool TRACE, bool CV, bool MOM> struct march_cells_kernel<MODE, TRACE, CV, MOM, true> {
    static constexpr void (*fn)(const MarchParams) = march_gen_kernel<MODE, TRACE, CV, MOM>;
};

template <bool GEN>
int launch_march_cells(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                       bool mom) {
    cudaStream_t st = (cudaStream_t)stream;
    if (trace) { blocks = 1; threads = 32; mom = false; }
    const size_t smem = march_smem(p, threads, kLaneCells);
#define DNSMC_L(M, T, CV_, O) \
    return march_launch_one(march_cells_kernel<M, T, CV_, O, GEN>::fn, blocks, threads, smem, st, p)
#define DNSMC_MODE(M)                                                                                  \
    if (trace) { if (cv) DNSMC_L(M, true, true, false); else DNSMC_L(M, true, false, false); }         \
    else if (cv) { if (mom) DNSMC_L(M, false, true, true); else DNSMC_L(M, false, true, false); }      \
    else DNSMC_L(M, false, false, false);
    switch (mode) {
        case MODE_GREY: DNSMC_MODE(MODE_GREY) break;
        case MODE_T: DNSMC_MODE(MODE_T) break;
        case MODE_TX: DNSMC_MODE(MODE_TX) break;
        default: break;
    }
#undef DNSMC_MODE
#undef DNSMC_L
    return (int)cudaErrorInvalidValue;
}

template <bool GEN>
int march_cells_occupancy(int mode, int threads, bool cv, bool mom, size_t smem) {
    int nb = 0;
#define DNSMC_O(M)                                                                                        \
    nb = cv ? (mom ? march_occupancy_one(march_cells_kernel<M, false, true, true, GEN>::fn, threads, smem)     \
                   : march_occupancy_one(march_cells_kernel<M, false, true, false, GEN>::fn, threads, smem))   \
            : march_occupancy_one(march_cells_kernel<M, false, false, false, GEN>::fn, threads, smem)
    if (mode == MODE_GREY) DNSMC_O(MODE_GREY);
    if (mode == MODE_T) DNSMC_O(MODE_T);
    if (mode == MODE_TX) DNSMC_O(MODE_TX);
#undef DNSMC_O
    return nb > 0 ? nb : 1;
}

}  // namespace dnsmc
