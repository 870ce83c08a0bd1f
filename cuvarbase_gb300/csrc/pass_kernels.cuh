// Pass kernels of the two-pass NFFT, templated on the transform lengths, and
// the device helpers they share with kernels.cu.
//
//   k_pass1<NG, L1>  one CTA per (curve, block of B columns).  Spreads the
//                    records of the neighbouring bins into NG padded
//                    L1 x B shared-memory tiles (shared-memory float atomics),
//                    runs the length-L1 column FFTs, applies the inter-pass
//                    twiddle exp(2 pi i q1 l2 / G) and writes the tile to the
//                    intermediate buffer (row-major, rows of G2).
//   k_pass2_gls<L2>  one CTA per (curve, block of R rows).  Loads R rows of
//                    the three grids, runs the length-L2 row FFTs and, in the
//                    same kernel, deconvolves the Gaussian window and
//                    evaluates the GLS power of every in-band frequency.
//   k_pass2_nfft<L2> the same for one grid, writing complex adjoint-NFFT
//                    values with the absolute-time phase.
#pragma once

#include <climits>
#include <cuda_runtime.h>

#include "fft.cuh"
#include "gls_math.cuh"
#include "kernels.cuh"

namespace cuvgls {

__device__ __forceinline__ void bin_ranges(const int *__restrict__ bins, int cb,
                                           int lo, int hi, int nb, int &a0,
                                           int &a1, int &b0, int &b1) {
    if (hi - lo + 1 >= nb) {
        a0 = bins[0]; a1 = bins[nb]; b0 = 0; b1 = 0;
        return;
    }
    const int s = cb + lo, e = cb + hi;
    if (s < 0) {
        a0 = bins[s + nb]; a1 = bins[nb]; b0 = bins[0]; b1 = bins[e + 1];
    } else if (e >= nb) {
        a0 = bins[s]; a1 = bins[nb]; b0 = bins[0]; b1 = bins[e - nb + 1];
    } else {
        a0 = bins[s]; a1 = bins[e + 1]; b0 = 0; b1 = 0;
    }
}

// Band index of FFT output q, or -1 when q is outside the centred band
// k' in [-h, nf - h).
__device__ __forceinline__ int band_index(long long q, int nf, int h, long long G) {
    if (q < nf - h) return (int)q;
    if (q >= G - h) return (int)(q - G);
    return INT_MIN;
}

// Position of the n-th (from 0) set bit of m; needs n < popc(m).
__device__ __forceinline__ int nth_set_bit(unsigned m, int n) {
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const int c = __popc(m & ((1u << w) - 1u));
        if (n >= c) { n -= c; m >>= w; pos += w; }
    }
    return pos;
}

// Stage A of the two-level column FFTs of a pass-1 tile (NG grids of B
// columns) that skips the units whose inputs are all zero.  Unit (g, i, c)
// transforms the elements i + LB k of column c of grid g; bit i of mAB
// (grids A and B) or mC (grid C) says that some row i + LB k holds a tap.
// A skipped unit's elements stay zero, which is their transform.  The
// remaining units are packed onto the lowest threads, so whole warps idle
// and leave their issue slots to the other CTAs of the SM.  With full masks
// this is the unit order of tile_fft2_a.
template <int L, int NG, int B, int GS, int NT>
__device__ __forceinline__ void tile_fft2_a_occ(float2 *__restrict__ buf,
                                                const float2 *__restrict__ twa, int tid,
                                                unsigned mAB, unsigned mC) {
    constexpr int LA = two_level_la(L);
    constexpr int LB = L / LA;
    static_assert(LA > 0 && LB <= 32, "two-level length with at most 32 residues");
    const int nAB = __popc(mAB), nC = NG == 3 ? __popc(mC) : 0;
    const int units = (NG == 3 ? 2 * nAB + nC : nAB) * B;
#pragma unroll 1
    for (int u = tid; u < units; u += NT) {
        const int c = u % B;
        int p = u / B, g = 0;
        unsigned mk = mAB;
        if (p >= nAB) {
            p -= nAB;
            g = 1;
            if (p >= nAB) { p -= nAB; g = 2; mk = mC; }
        }
        const int i = nth_set_bit(mk, p);
        const int base = c + g * GS;
        float2 x[LA];
#pragma unroll
        for (int k = 0; k < LA; ++k) x[k] = buf[base + phys2_ik<L>(i, k) * B];
        fft2_stage_a_regs<L>(x, twa, i);
#pragma unroll
        for (int qa = 0; qa < LA; ++qa) buf[base + phys2_ik<L>(i, qa) * B] = x[qa];
    }
}

// Exclusive scan of c[0..n) in place by the whole CTA of NT threads (each
// thread a run of ceil(n / NT) consecutive entries), c[n] = total; ws holds
// the 32 warp sums.  Ends with a barrier.
template <int NT>
__device__ __forceinline__ void block_scan_counts(int *c, int n, int *ws, int tid) {
    static_assert(NT % 32 == 0 && NT <= 1024, "whole warps");
    constexpr int NW = NT / 32;
    const int per = (n + NT - 1) / NT;
    const int i0 = min(tid * per, n), i1 = min(i0 + per, n);
    int sum = 0;
    for (int i = i0; i < i1; ++i) sum += c[i];
    const int lane = tid & 31, wid = tid >> 5;
    int inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int v = (lane < NW) ? ws[lane] : 0;
        int iv = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, iv, o);
            if (lane >= o) iv += y;
        }
        if (lane < NW) ws[lane] = iv - v;
        if (lane == NW - 1) c[n] = iv;
    }
    __syncthreads();
    int run = ws[wid] + inc - sum;
    for (int i = i0; i < i1; ++i) {
        const int v = c[i];
        c[i] = run;
        run += v;
    }
    __syncthreads();
}

// A record staged by pass 1: row << 16 | column of its cell, offset in the
// cell, and its values (grids A and B, or grid C twice).
struct StagedRec {
    int rc;
    float frac;
    float2 v0, v1;
};
static_assert(sizeof(StagedRec) == kStageRecBytes, "staged record size");

// One pass-1 CTA: column block blockIdx.x of curve blockIdx.y (the body of
// both pass-1 kernels below).
template <int NG, int L1>
__device__ __forceinline__ void pass1_body(const DevCurve *__restrict__ cvs,
                                           const RecAB *__restrict__ recAB,
                                           const RecC *__restrict__ recC,
                                           const int *__restrict__ binsAB,
                                           const int *__restrict__ binsC,
                                           float2 *__restrict__ inter, const Plan &p) {
    constexpr int B = pass1_cols(NG, L1);
    constexpr int NT = pass1_threads(NG, L1);
    constexpr int GS = tile_len(L1) * B;
    constexpr int TILE = NG * GS;
    constexpr int NTW = fft_table_len(L1);
    constexpr int NSR = pass1_stage_recs(NG, L1);
    // staged records follow the tile (and the Stockham table)
    constexpr int STAGE = TILE + (two_level_la(L1) ? 0 : NTW);
    extern __shared__ __align__(16) float2 sm[];
    float2 *tile = sm;
    const int tid = threadIdx.x;
    const int cb = blockIdx.x;
    const DevCurve cv = cvs[blockIdx.y];
    const int c0 = cb * B;
    const int G2 = p.G2, m = p.m;
    // FFT table: read through the read-only cache (two-level lengths) or
    // staged in shared memory (Stockham lengths)
    const float2 *tws = p.st1;
    if constexpr (two_level_la(L1) == 0) {
        float2 *t = tile + TILE;
        for (int i = tid; i < NTW; i += NT) t[i] = p.st1[i];
        tws = t;
    }
    {
        float4 *t4 = reinterpret_cast<float4 *>(tile);  // 16-byte aligned
        for (int i = tid; i < TILE / 2; i += NT) t4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if ((TILE & 1) && tid == 0) tile[TILE - 1] = make_float2(0.f, 0.f);
    }

    // Spreading.  The records of the neighbouring bins (grids A and B share
    // the x-position records, grid C has its own at 2x positions; each
    // carries its cell as row and column) are staged in shared memory NSR at
    // a time, one batch of coalesced loads per round.  Then one work item per
    // (staged record, column of this block), or the gather below.
    const int lo = -((m + B - 1) / B), hi = (B + m - 2) / B;
    int a0, a1, b0, b1, e0 = 0, e1 = 0, f0 = 0, f1 = 0;
    bin_ranges(binsAB + cv.bin_off, cb, lo, hi, p.nb, a0, a1, b0, b1);
    const int nab = (a1 - a0) + (b1 - b0);
    int nc = 0;
    if (NG == 3) {
        bin_ranges(binsC + cv.bin_off, cb, lo, hi, p.nb, e0, e1, f0, f1);
        nc = (e1 - e0) + (f1 - f0);
    }
    const RecAB *rab = recAB + cv.rec_off;
    const RecC *rcc = recC + cv.rec_off;
    StagedRec *st = reinterpret_cast<StagedRec *>(sm + STAGE);
    const int ntot = nab + nc;
    // Dense column blocks of the long Stockham tiles (at least one record per
    // row of the tile) are spread by gather: the staged records are sorted
    // by the row they land in (integer shared-memory atomics and a scan),
    // then each thread sums the taps of whole rows in registers and adds
    // them to the tile with plain stores; no float atomics, which serialise
    // when several records hit the same cells.
    constexpr bool GATHER = pass1_gather(NG, L1);
    int *rowcnt = reinterpret_cast<int *>(st + NSR);  // L1 + 1 (gather tiles)
    int *bucket = rowcnt + L1 + 1;                      // NSR
    int *wsum = bucket + NSR;                           // 32
    const bool dense = GATHER && ntot >= L1;
    // Two-level column FFTs: occ[kind * 32 + i] is set when a tap of that
    // record kind (0: A and B, 1: C) lands in a row congruent to i modulo
    // LB, so stage A can skip the all-zero units; the dense path does not
    // track it and transforms every unit.
    constexpr int LA1 = two_level_la(L1);
    constexpr int LB1 = LA1 ? L1 / LA1 : 1;
    unsigned char *occ = reinterpret_cast<unsigned char *>(st + NSR) +
                         (GATHER ? pass1_gather_bytes(L1, NSR) : 0);  // kOccBytes
    if (LA1 && tid < kOccBytes) occ[tid] = 0;  // before the first round's barrier
    if (dense) {  // uniform over the CTA
        for (int i = tid; i <= L1; i += NT) rowcnt[i] = 0;
        __syncthreads();  // counts zeroed before the first round's atomics
    }
    // staged form of record ri of this block's window (AB records first)
    auto load_rec = [&](int ri) {
        StagedRec r;
        if (ri < nab) {
            const int k = ri < (a1 - a0) ? a0 + ri : b0 + (ri - (a1 - a0));
            const RecAB q = rab[k];
            r.rc = q.rc; r.frac = q.frac; r.v0 = q.a; r.v1 = q.b;
        } else {
            const int rj = ri - nab;
            const int k = rj < (e1 - e0) ? e0 + rj : f0 + (rj - (e1 - e0));
            const RecC q = rcc[k];
            r.rc = q.rc; r.frac = q.frac; r.v0 = q.c; r.v1 = q.c;
        }
        return r;
    };
    for (int base = 0;; base += NSR) {
        const int cnt = min(NSR, ntot - base);
        if (GATHER && dense) {
            constexpr int RPT = (NSR + NT - 1) / NT;
            // 1. stage the round's records with the row each lands in for
            //    this block (one wrap decision per record: with G2 >= 2m + B
            //    the per-column wraps agree wherever a tap is inside the
            //    window), the offset x of its tap in column c0 kept in rc,
            //    and its rank within the row; records without a tap here
            //    are dropped
            int myrow[RPT], myrank[RPT];
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                const int j = tid + q * NT;
                myrow[q] = -1;
                myrank[q] = 0;
                if (j < cnt) {
                    StagedRec r = load_rec(base + j);
                    const int ck = r.rc & 0xFFFF;
                    int row = r.rc >> 16, x = c0 - ck;
                    if (x + B - 1 < 1 - m) { x += G2; row += 1; }
                    else if (x > m) { x -= G2; row -= 1; }
                    if (x + B - 1 >= 1 - m && x <= m) {
                        if (row < 0) row += L1;
                        else if (row >= L1) row -= L1;
                        r.rc = x;
                        st[j] = r;
                        myrow[q] = row;
                        myrank[q] = atomicAdd(&rowcnt[row], 1);
                    }
                }
            }
            __syncthreads();  // counts (and, first time, the zeroed tile)
            // 2. row offsets
            block_scan_counts<NT>(rowcnt, L1, wsum, tid);
            // 3. records in row order
#pragma unroll
            for (int q = 0; q < RPT; ++q)
                if (myrow[q] >= 0) {
                    const int at = rowcnt[myrow[q]] + myrank[q];
                    if ((unsigned)at < (unsigned)cnt) bucket[at] = tid + q * NT;
                }
            __syncthreads();
            // 4. whole rows per thread: taps summed in registers
            for (int r = tid; r < L1; r += NT) {
                float2 aA[B], aB[B], aC[B];
#pragma unroll
                for (int cc = 0; cc < B; ++cc) {
                    aA[cc] = make_float2(0.f, 0.f);
                    aB[cc] = make_float2(0.f, 0.f);
                    aC[cc] = make_float2(0.f, 0.f);
                }
                // (bounds: offsets within the round's records, indices of
                // staged records)
                const int g0 = max(rowcnt[r], 0), g1 = min(rowcnt[r + 1], cnt);
                for (int e = g0; e < g1; ++e) {
                    const int j = bucket[e];
                    if ((unsigned)j >= (unsigned)cnt) continue;
                    const StagedRec rec = st[j];
                    const bool ab = base + j < nab;
#pragma unroll
                    for (int cc = 0; cc < B; ++cc) {
                        const int d = rec.rc + cc;
                        if (d < 1 - m || d > m) continue;
                        const float dd = (float)d - rec.frac;
                        const float wg = win_tap(dd, p);
                        if (ab) {
                            aA[cc] = make_float2(fmaf(rec.v0.x, wg, aA[cc].x),
                                                 fmaf(rec.v0.y, wg, aA[cc].y));
                            if (NG == 3)
                                aB[cc] = make_float2(fmaf(rec.v1.x, wg, aB[cc].x),
                                                     fmaf(rec.v1.y, wg, aB[cc].y));
                        } else {
                            aC[cc] = make_float2(fmaf(rec.v0.x, wg, aC[cc].x),
                                                 fmaf(rec.v0.y, wg, aC[cc].y));
                        }
                    }
                }
                float2 *rp = tile + phys2<L1>(r) * B;
#pragma unroll
                for (int cc = 0; cc < B; ++cc) {
                    rp[cc] = cadd(rp[cc], aA[cc]);
                    if (NG == 3) {
                        rp[GS + cc] = cadd(rp[GS + cc], aB[cc]);
                        rp[2 * GS + cc] = cadd(rp[2 * GS + cc], aC[cc]);
                    }
                }
            }
            __syncthreads();  // rows summed before the counts are reset
            for (int i = tid; i <= L1; i += NT) rowcnt[i] = 0;
        } else {
            for (int j = tid; j < cnt; j += NT) st[j] = load_rec(base + j);
            __syncthreads();  // staged records (and, first time, the zeroed tile)
            for (int it = tid; it < cnt * B; it += NT) {
                const int j = it / B, cc = it % B;
                const StagedRec r = st[j];
                const bool ab = base + j < nab;
                float2 *t0 = ab ? tile : tile + 2 * GS;
                // tap d of this record lands in column c0 + cc (modulo the row wrap)
                const int ck = r.rc & 0xFFFF, rk = r.rc >> 16;
                int d = c0 + cc - ck, row = rk;
                if (d < 1 - m) { d += G2; row += 1; }
                else if (d > m) { d -= G2; row -= 1; }
                if (d < 1 - m || d > m) continue;
                if (row < 0) row += L1;
                else if (row >= L1) row -= L1;
                if constexpr (LA1 > 0) occ[(ab ? 0 : 32) + row % LB1] = 1;
                const float dd = (float)d - r.frac;
                const float wg = win_tap(dd, p);
                float2 *cp = t0 + phys2<L1>(row) * B + cc;
                atomicAdd(&cp->x, r.v0.x * wg);
                atomicAdd(&cp->y, r.v0.y * wg);
                if (NG == 3 && ab) {
                    atomicAdd(&cp[GS].x, r.v1.x * wg);
                    atomicAdd(&cp[GS].y, r.v1.y * wg);
                }
            }
        }
        __syncthreads();  // the round is spread before it is overwritten
        if (base + NSR >= ntot) break;
    }

    // The intermediate of grid g is stored column-block-major,
    // I_g[cb][q1][c] (c fastest), so this CTA writes one contiguous block of
    // L1 B elements per grid.  The inter-pass twiddle
    // exp(2 pi i q1 (c0 + c) / G) comes from the plan table in the same order.
    const long long blk = (long long)cb * L1 * B;
    float2 *dst = inter + cv.inter_off + blk;
    const float2 *itw = p.itw + blk;
    const long long G = p.G;
    // vectors (g, c): base g * GS + c, element stride B
    if constexpr (two_level_la(L1) > 0) {
        // stage B stores straight to the intermediate: unit (g, c, qa) owns
        // outputs q1 = qa + LA qb, and consecutive threads run consecutive
        // (c, qa), so a warp writes contiguous runs of whole q1 rows
        constexpr int LA = two_level_la(L1), LB = L1 / LA;
        constexpr unsigned kAll = LB == 32 ? 0xFFFFFFFFu : (1u << LB) - 1u;
        unsigned mAB = kAll, mC = kAll;
        if (!dense) {  // uniform over the CTA; flags final after the last round's barrier
            const int lane = tid & 31;
            mAB = __ballot_sync(0xFFFFFFFFu, lane < LB && occ[lane] != 0);
            mC = __ballot_sync(0xFFFFFFFFu, lane < LB && occ[32 + lane] != 0);
        }
        tile_fft2_a_occ<L1, NG, B, GS, NT>(tile, tws, tid, mAB, mC);
        __syncthreads();
        float2 y[LB];
        int g, c, qa;
        if (tile_fft2_b<L1, NG * B, B, 1, GS, B, NT>(tile, tid, y, g, c, qa)) {
            // per-thread base pointers, then compile-time offsets qb La B
            // (one address computation per thread, not one per element)
            const int e0 = qa * B + c;
            float2 *d = dst + g * G + e0;
            const float2 *w = itw + e0;
#pragma unroll
            for (int qb = 0; qb < LB; ++qb) d[qb * LA * B] = cmul(y[qb], __ldg(w + qb * LA * B));
        }
    } else {
        tile_fft_any<L1, NG * B, B, 1, GS, B, NT>(tile, tws, tid);
#pragma unroll 2
        for (int e = tid; e < L1 * B; e += NT) {
            const int q1 = e / B, c = e % B;
            const float2 w = __ldg(itw + e);
            const int src = phys2<L1>(q1) * B + c;
#pragma unroll
            for (int g = 0; g < NG; ++g) dst[g * G + e] = cmul(tile[g * GS + src], w);
        }
    }
}

// Pass 1 with the compiler's own register choice ...
template <int NG, int L1>
__global__ void __launch_bounds__(pass1_threads(NG, L1))
k_pass1(const DevCurve *__restrict__ cvs, const RecAB *__restrict__ recAB,
        const RecC *__restrict__ recC, const int *__restrict__ binsAB,
        const int *__restrict__ binsC, float2 *__restrict__ inter, Plan p) {
    pass1_body<NG, L1>(cvs, recAB, recC, binsAB, binsC, inter, p);
}

// ... and, for the tiles whose smaller staging fits one more CTA per SM
// (pass1_small_stage), bound to that many CTAs per SM.  A minimum of one CTA
// per SM is not the same as no bound: it lets the compiler spend up to 255
// registers (pass 1 of rows of 400: 60 -> 110 registers, half the CTAs).
template <int NG, int L1>
__global__ void __launch_bounds__(pass1_threads(NG, L1), pass1_min_ctas(NG, L1))
k_pass1_occ(const DevCurve *__restrict__ cvs, const RecAB *__restrict__ recAB,
            const RecC *__restrict__ recC, const int *__restrict__ binsAB,
            const int *__restrict__ binsC, float2 *__restrict__ inter, Plan p) {
    pass1_body<NG, L1>(cvs, recAB, recC, binsAB, binsC, inter, p);
}

template <int NG, int L2, int R, int NT, int LDS, int B>
__device__ __forceinline__ void load_rows_b(float2 *tile, const float2 *__restrict__ src,
                                            int G1, long long G, int rb, int tid) {
    // Consecutive threads fill consecutive element pairs of one tile row
    // (conflict-free shared stores); each pair is a 16-byte global load.
    constexpr int PR = L2 / 2;          // element pairs per row
    static_assert(B % 2 == 0, "B must be even");
#pragma unroll 4
    for (int e = tid; e < NG * R * PR; e += NT) {
        const int pr = e % PR, v = e / PR;
        const int g = v / R, r = v - g * R;
        const int l2 = 2 * pr;
        const int cb = l2 / B, c = l2 % B;
        const float4 val = *reinterpret_cast<const float4 *>(
            src + g * G + ((long long)cb * G1 + (long long)rb * R + r) * B + c);
        float2 *d = tile + v * LDS;
        d[phys2<L2>(l2)] = make_float2(val.x, val.y);
        d[phys2<L2>(l2 + 1)] = make_float2(val.z, val.w);
    }
}

// Rows rb R .. rb R + R - 1 of NG grids, transformed along the row (length
// L2) into the padded tile; ends with a barrier.  With a two-level split
// whose LB is a multiple of B, stage A reads its inputs straight from the
// intermediate: unit (g, r, i = ih B + c) takes elements i + LB k, all in
// column block ih + (LB / B) k at column c, and consecutive threads run
// consecutive (c, r), so a warp reads whole R x B blocks.  Otherwise the
// rows are loaded into the tile first.
template <int NG, int L2, int R, int NT, int LDS, int B>
__device__ __forceinline__ void rows_fft_b(float2 *tile, const float2 *__restrict__ src,
                                           const float2 *__restrict__ tab, int G1, long long G,
                                           int rb, int tid) {
    constexpr int LA = two_level_la(L2);
    if constexpr (LA > 0 && (L2 / LA) % B == 0) {
        constexpr int LB = L2 / LA, IH = LB / B;
        const int kstride = IH * G1 * B;  // elements between column blocks ih and ih + IH
#pragma unroll 1
        for (int u = tid; u < NG * R * LB; u += NT) {
            const int c = u % B;
            int t = u / B;
            const int r = t % R;
            t /= R;
            const int ih = t % IH, g = t / IH;
            const float2 *s = src + g * G + (ih * G1 + rb * R + r) * B + c;
            float2 x[LA];
#pragma unroll
            for (int k = 0; k < LA; ++k) x[k] = __ldg(s + k * kstride);
            const int i = ih * B + c;
            fft2_stage_a_regs<L2>(x, tab, i);
            float2 *d = tile + (g * R + r) * LDS;
#pragma unroll
            for (int qa = 0; qa < LA; ++qa) d[phys2_ik<L2>(i, qa)] = x[qa];
        }
        __syncthreads();
        tile_fft2_b_inplace<L2, NG * R, 1, 0, LDS, 1, NT>(tile, tid);
    } else {
        load_rows_b<NG, L2, R, NT, LDS, B>(tile, src, G1, G, rb, tid);
        const float2 *tws = tab;
        if constexpr (LA == 0) {
            float2 *t = tile + NG * R * LDS;
            for (int i = tid; i < fft_table_len(L2); i += NT) t[i] = tab[i];
            tws = t;
        }
        __syncthreads();
        tile_fft_any<L2, NG * R, 1, 0, LDS, 1, NT>(tile, tws, tid);
    }
}

template <int NG, int L2, int R, int NT, int LDS>
__device__ __forceinline__ void rows_fft(float2 *tile, const float2 *__restrict__ src,
                                         const float2 *__restrict__ tab, int G1, long long G,
                                         int B, int rb, int tid) {
    if (B == 8) rows_fft_b<NG, L2, R, NT, LDS, 8>(tile, src, tab, G1, G, rb, tid);
    else if (B == 4) rows_fft_b<NG, L2, R, NT, LDS, 4>(tile, src, tab, G1, G, rb, tid);
    else rows_fft_b<NG, L2, R, NT, LDS, 2>(tile, src, tab, G1, G, rb, tid);
}

// Deconvolution + GLS power of every in-band frequency of the R rows of a
// pass-2 tile.  BEST: also fold each valid power into the curve's best key
// (power bits << 32 | ~index, one atomicMax per warp; the caller guarantees
// full warps), and out == nullptr skips the powers themselves.  Chosen once
// per CTA, so the plain path carries no per-frequency cost for it.
template <bool BEST, bool ES, int L2, int R, int NT, int LDS>
__device__ __forceinline__ void gls_epilogue(const float2 *tile, const DevCurve &cv,
                                             float *__restrict__ out, const GlsParams &gp,
                                             const Plan &p, int rb, int tid) {
    const int G = (int)p.G;  // < 2^23
    const int G1 = p.G1;
    const int nf = cv.nf, h = nf / 2;
    const int lo_end = nf - h, hi_start = G - h;
    float *outc = (!BEST || out) ? out + cv.out_off + h : nullptr;
    unsigned long long key = 0;
    const unsigned ibase = (unsigned)(cv.best_off + h);
#pragma unroll 2
    for (int e = tid; e < R * L2; e += NT) {
        const int r = e % R, q2 = e / R;
        const int q = rb * R + r + G1 * q2;
        int kp;
        if (q < lo_end) kp = q;
        else if (q >= hi_start) kp = q - G;
        else continue;
        const float D = win_deconv<ES>(kp, p);
        const int o = phys2<L2>(q2);
        const float2 A = tile[r * LDS + o];
        const float2 Bv = tile[(R + r) * LDS + o];
        const float2 Cv = tile[(2 * R + r) * LDS + o];
        const float P = gls_from_sums<float>(
            A.x * D, A.y * D, Bv.x * D, Bv.y * D, Cv.x * D, Cv.y * D, gp.mode,
            gp.reg, cv.w_sum, cv.yw_sum, cv.ybar, cv.yy_inv);
        if (!BEST || outc) outc[kp] = P;
        if (BEST && P >= 0.f) {  // valid powers only (invalid ones are -1)
            const unsigned long long k =
                ((unsigned long long)__float_as_uint(P) << 32) |
                (0xFFFFFFFFu - (ibase + (unsigned)kp));
            key = k > key ? k : key;
        }
    }
    if (BEST) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long v = __shfl_xor_sync(0xffffffffu, key, o);
            key = v > key ? v : key;
        }
        if ((tid & 31) == 0 && key != 0) atomicMax(gp.best + cv.best_slot, key);
    }
}

// Floating-mean GLS finish of a pass-2 tile (mode 1) with two frequencies
// per thread evaluated together as packed FP32x2 arithmetic: lane 0 is row
// element q2, lane 1 element q2 + NT / R of the same row.  Same quantities
// as gls_from_sums (2x2 normal equations, invalid -> -1); BEST as in
// gls_epilogue.
template <bool BEST, bool ES, int L2, int R, int NT, int LDS>
__device__ __forceinline__ void gls_epilogue_fm2(const float2 *tile, const DevCurve &cv,
                                                 float *__restrict__ out, const GlsParams &gp,
                                                 const Plan &p, int rb, int tid) {
    static_assert(NT % R == 0 && NT % 32 == 0, "one row per thread, full warps");
    constexpr int QS = NT / R;
    const int G = (int)p.G;  // < 2^23
    const int G1 = p.G1;
    const int nf = cv.nf, h = nf / 2;
    const int lo_end = nf - h, hi_start = G - h;
    float *outc = (!BEST || out) ? out + cv.out_off + h : nullptr;
    unsigned long long key = 0;
    const unsigned ibase = (unsigned)(cv.best_off + h);
    auto keep = [&](float P, int k) {  // fold a valid power into the best key
        if (P >= 0.f) {
            const unsigned long long kk = ((unsigned long long)__float_as_uint(P) << 32) |
                                          (0xFFFFFFFFu - (ibase + (unsigned)k));
            key = kk > key ? kk : key;
        }
    };
    const int r = tid % R, q20 = tid / R;
    const float2 *tA = tile + r * LDS, *tB = tile + (R + r) * LDS, *tC = tile + (2 * R + r) * LDS;
    const float2 dc1 = make_float2(p.dc1, p.dc1), dc2 = make_float2(p.dc2, p.dc2);
    const float2 nyw = make_float2(-cv.yw_sum, -cv.yw_sum);
    const float hw0 = 0.5f * cv.w_sum + gp.reg;
    const float2 hw = make_float2(hw0, hw0), half = make_float2(0.5f, 0.5f);
    const float2 mhalf = make_float2(-0.5f, -0.5f), mtwo = make_float2(-2.f, -2.f);
    const float2 pn = make_float2(cv.yy_inv, cv.yy_inv);
#pragma unroll 1
    for (int q2a = q20; q2a < L2; q2a += 2 * QS) {
        const int q2b = q2a + QS;
        const int qa = rb * R + r + G1 * q2a, qb = qa + G1 * QS;
        const bool ina = qa < lo_end || qa >= hi_start;
        const bool inb = q2b < L2 && (qb < lo_end || qb >= hi_start);
        if (!ina && !inb) continue;
        const int ka = qa < lo_end ? qa : qa - G, kb = qb < lo_end ? qb : qb - G;
        const int oa = phys2<L2>(q2a), ob = phys2<L2>(q2b < L2 ? q2b : q2a);
        const float2 A0 = tA[oa], A1 = tA[ob], B0 = tB[oa], B1 = tB[ob];
        const float2 C0 = tC[oa], C1 = tC[ob];
        // deconvolution per lane: the Gaussian's exp(b (pi k' / G)^2) / sqrt(pi b),
        // or the plan's table
        float2 D;
        if constexpr (ES) {
            // (an out-of-band lane reads entry 0: |k'| <= G / 2 only in band)
            D = make_float2(__ldg(p.dtab + (ina ? abs(ka) : 0)),
                            __ldg(p.dtab + (inb ? abs(kb) : 0)));
        } else {
            const float2 kf = make_float2((float)ka, (float)kb);
            const float2 ex = __fmul2_rn(__fmul2_rn(kf, kf), dc1);
            D = __fmul2_rn(make_float2(__expf(ex.x), __expf(ex.y)), dc2);
        }
        const float2 YCh = __fmul2_rn(make_float2(A0.x, A1.x), D);
        const float2 YSh = __fmul2_rn(make_float2(A0.y, A1.y), D);
        const float2 C = __fmul2_rn(make_float2(B0.x, B1.x), D);
        const float2 S = __fmul2_rn(make_float2(B0.y, B1.y), D);
        const float2 C2 = __fmul2_rn(make_float2(C0.x, C1.x), D);
        const float2 S2 = __fmul2_rn(make_float2(C0.y, C1.y), D);
        const float2 mC = make_float2(-C.x, -C.y), mS = make_float2(-S.x, -S.y);
        const float2 YC = __ffma2_rn(nyw, C, YCh);
        const float2 YS = __ffma2_rn(nyw, S, YSh);
        const float2 CC = __ffma2_rn(mC, C, __ffma2_rn(half, C2, hw));
        const float2 SS = __ffma2_rn(mS, S, __ffma2_rn(mhalf, C2, hw));
        const float2 CS = __ffma2_rn(mC, S, __fmul2_rn(half, S2));
        const float2 det = __ffma2_rn(make_float2(-CS.x, -CS.y), CS, __fmul2_rn(CC, SS));
        const float2 a = __ffma2_rn(__fmul2_rn(mtwo, YS), CS, __fmul2_rn(YC, SS));
        const float2 num = __ffma2_rn(YC, a, __fmul2_rn(__fmul2_rn(YS, YS), CC));
        const float2 P = __fmul2_rn(make_float2(__fdividef(num.x, det.x),
                                                __fdividef(num.y, det.y)), pn);
        const float Pa = (P.x >= 0.f && !isinf(P.x)) ? P.x : -1.f;
        const float Pb = (P.y >= 0.f && !isinf(P.y)) ? P.y : -1.f;
        if (!BEST || outc) {
            if (ina) outc[ka] = Pa;
            if (inb) outc[kb] = Pb;
        }
        if (BEST) {
            if (ina) keep(Pa, ka);
            if (inb) keep(Pb, kb);
        }
    }
    if (BEST) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long v = __shfl_xor_sync(0xffffffffu, key, o);
            key = v > key ? v : key;
        }
        if ((tid & 31) == 0 && key != 0) atomicMax(gp.best + cv.best_slot, key);
    }
}

template <int L2>
__global__ void __launch_bounds__(pass2_threads(3, L2))
k_pass2_gls(const DevCurve *__restrict__ cvs, const float2 *__restrict__ inter,
            float *__restrict__ out, Plan p, GlsParams gp) {
    constexpr int R = pass2_rows(3, L2);
    constexpr int NT = pass2_threads(3, L2);
    static_assert(NT % 32 == 0, "the best-power reduction needs full warps");
    constexpr int LDS = row_stride(L2);
    extern __shared__ __align__(16) float2 sm[];
    float2 *tile = sm;
    const int tid = threadIdx.x, rb = blockIdx.x;
    const DevCurve cv = cvs[blockIdx.y];
    const int G1 = p.G1;
    rows_fft<3, L2, R, NT, LDS>(tile, inter + cv.inter_off, p.st2, G1, p.G, p.B, rb, tid);
    // The packed finish is compiled only into the 4-row tiles (rows of 256 to
    // 1024: 256 threads at up to 64 registers, 4 CTAs per SM either way).
    // In the 16-row tiles of short rows (480 threads) its extra registers
    // would cost a CTA per SM (rows of 80: 37 -> 42 registers, 3 -> 2 CTAs,
    // pass 2 43 -> 56 ms on 200,000 curves).
    // (window and output kind chosen once per CTA: each finish is compiled
    // for one window, with no per-frequency branch)
    const bool es = p.win == kWinES;
    if constexpr (R == 4) {
        if (gp.mode == 1) {
            if (es) {
                if (gp.best) gls_epilogue_fm2<true, true, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
                else gls_epilogue_fm2<false, true, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
            } else {
                if (gp.best) gls_epilogue_fm2<true, false, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
                else gls_epilogue_fm2<false, false, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
            }
            return;
        }
    }
    if (es) {
        if (gp.best) gls_epilogue<true, true, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
        else gls_epilogue<false, true, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
    } else {
        if (gp.best) gls_epilogue<true, false, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
        else gls_epilogue<false, false, L2, R, NT, LDS>(tile, cv, out, gp, p, rb, tid);
    }
}

// Adjoint-NFFT finish of a pass-2 tile: deconvolution and the phase of the
// absolute time origin, complex output per in-band frequency.
template <bool ES, int L2, int R, int NT, int LDS>
__device__ __forceinline__ void nfft_finish(const float2 *tile, const DevCurve &cv,
                                            float2 *__restrict__ out,
                                            const float4 *__restrict__ aux, const Plan &p,
                                            int rb, int tid) {
    const float4 ax = aux[cv.aux];
    const float2 base = make_float2(ax.x, ax.y);
    const long long G = p.G;
    const int G1 = p.G1;
    const int nf = cv.nf, h = nf / 2;
    for (int e = tid; e < R * L2; e += NT) {
        const int r = e % R, q2 = e / R;
        const int kp = band_index((long long)(rb * R + r) + (long long)G1 * q2, nf, h, G);
        if (kp == INT_MIN) continue;
        const float kf = (float)kp;
        const float D = win_deconv<ES>(kp, p);
        // frac(k' alpha) with alpha = hi + lo and k' alpha_hi split exactly
        const float pr = kf * ax.z;
        const float er = fmaf(kf, ax.z, -pr);
        const float th = (pr - rintf(pr)) + (er + kf * ax.w);
        float s, c;
        sincospif(2.0f * th, &s, &c);
        const float2 ph = cmul(base, make_float2(c, s));
        out[cv.out_off + kp + h] = cmul(cscale(tile[r * LDS + phys2<L2>(q2)], D), ph);
    }
}

template <int L2>
__global__ void __launch_bounds__(pass2_threads(1, L2))
k_pass2_nfft(const DevCurve *__restrict__ cvs, const float2 *__restrict__ inter,
             float2 *__restrict__ out, const float4 *__restrict__ aux, Plan p) {
    constexpr int R = pass2_rows(1, L2);
    constexpr int NT = pass2_threads(1, L2);
    constexpr int LDS = row_stride(L2);
    extern __shared__ __align__(16) float2 sm[];
    float2 *tile = sm;
    const int tid = threadIdx.x, rb = blockIdx.x;
    const DevCurve cv = cvs[blockIdx.y];
    const int G1 = p.G1;
    rows_fft<1, L2, R, NT, LDS>(tile, inter + cv.inter_off, p.st2, G1, p.G, p.B, rb, tid);

    if (p.win == kWinES) nfft_finish<true, L2, R, NT, LDS>(tile, cv, out, aux, p, rb, tid);
    else nfft_finish<false, L2, R, NT, LDS>(tile, cv, out, aux, p, rb, tid);
}

// ---- launch templates (explicitly instantiated in the inst_*.cu files) ----
// Raise a kernel's dynamic shared-memory limit to `bytes`.  `done` is the
// caller's per-kernel cache (one per device): every length instantiation has
// its own, because instantiations share a function type but not attributes.
template <typename K>
static cudaError_t allow_smem(K kernel, size_t bytes, size_t (&done)[64]) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (bytes <= 48 * 1024 || bytes <= done[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes);
    if (e == cudaSuccess) done[dev] = bytes;
    return e;
}

template <int NG, int L1>
cudaError_t launch_pass1_t(const DevCurve *cv, int n_curves, const RecAB *recAB,
                           const RecC *recC, const int *binsAB, const int *binsC,
                           float2 *inter, const Plan &p, cudaStream_t s) {
    static size_t done[64] = {0};  // per instantiation
    const size_t smem = (size_t)pass1_smem(NG, L1, p.G);
    dim3 grid(p.G2 / pass1_cols(NG, L1), n_curves);
    if constexpr (pass1_small_stage(NG, L1)) {
        cudaError_t e = allow_smem(k_pass1_occ<NG, L1>, smem, done);
        if (e != cudaSuccess) return e;
        k_pass1_occ<NG, L1><<<grid, pass1_threads(NG, L1), smem, s>>>(cv, recAB, recC, binsAB,
                                                                        binsC, inter, p);
    } else {
        cudaError_t e = allow_smem(k_pass1<NG, L1>, smem, done);
        if (e != cudaSuccess) return e;
        k_pass1<NG, L1><<<grid, pass1_threads(NG, L1), smem, s>>>(cv, recAB, recC, binsAB,
                                                                    binsC, inter, p);
    }
    return cudaGetLastError();
}

template <int L2>
cudaError_t launch_pass2_gls_t(const DevCurve *cv, int n_curves, const float2 *inter,
                               float *out, const Plan &p, GlsParams g, cudaStream_t s) {
    static size_t done[64] = {0};  // per instantiation
    cudaError_t e = allow_smem(k_pass2_gls<L2>, (size_t)pass2_smem(3, L2), done);
    if (e != cudaSuccess) return e;
    dim3 grid(p.G1 / pass2_rows(3, L2), n_curves);
    k_pass2_gls<L2><<<grid, pass2_threads(3, L2), (size_t)pass2_smem(3, L2), s>>>(
        cv, inter, out, p, g);
    return cudaGetLastError();
}

template <int L2>
cudaError_t launch_pass2_nfft_t(const DevCurve *cv, int n_curves, const float2 *inter,
                                float2 *out, const float4 *aux, const Plan &p,
                                cudaStream_t s) {
    static size_t done[64] = {0};  // per instantiation
    cudaError_t e = allow_smem(k_pass2_nfft<L2>, (size_t)pass2_smem(1, L2), done);
    if (e != cudaSuccess) return e;
    dim3 grid(p.G1 / pass2_rows(1, L2), n_curves);
    k_pass2_nfft<L2><<<grid, pass2_threads(1, L2), (size_t)pass2_smem(1, L2), s>>>(
        cv, inter, out, aux, p);
    return cudaGetLastError();
}

// Load the pass kernels of a length now (CUDA loads kernels lazily, at
// their first launch, which would otherwise land in the first batch of a new
// plan class: a stall of milliseconds in a serving loop).
template <int NG, int L1>
cudaError_t preload_pass1_t() {
    cudaFuncAttributes a;
    if constexpr (pass1_small_stage(NG, L1)) return cudaFuncGetAttributes(&a, k_pass1_occ<NG, L1>);
    else return cudaFuncGetAttributes(&a, k_pass1<NG, L1>);
}
template <int L2>
cudaError_t preload_pass2_t(int ng) {
    cudaFuncAttributes a;
    return ng == 3 ? cudaFuncGetAttributes(&a, k_pass2_gls<L2>)
                   : cudaFuncGetAttributes(&a, k_pass2_nfft<L2>);
}

#define CUVGLS_INSTANTIATE_ROW_LEN(L)                                               \
    template cudaError_t launch_pass2_gls_t<L>(const DevCurve *, int, const float2 *, \
                                               float *, const Plan &, GlsParams,     \
                                               cudaStream_t);                        \
    template cudaError_t launch_pass2_nfft_t<L>(const DevCurve *, int, const float2 *, \
                                                float2 *, const float4 *, const Plan &, \
                                                cudaStream_t);                       \
    template cudaError_t preload_pass2_t<L>(int);

#define CUVGLS_INSTANTIATE_LEN(L)                                                   \
    template cudaError_t launch_pass1_t<3, L>(const DevCurve *, int, const RecAB *, \
                                              const RecC *, const int *, const int *, \
                                              float2 *, const Plan &, cudaStream_t); \
    template cudaError_t launch_pass1_t<1, L>(const DevCurve *, int, const RecAB *, \
                                              const RecC *, const int *, const int *, \
                                              float2 *, const Plan &, cudaStream_t); \
    template cudaError_t launch_pass2_gls_t<L>(const DevCurve *, int, const float2 *, \
                                               float *, const Plan &, GlsParams,     \
                                               cudaStream_t);                        \
    template cudaError_t launch_pass2_nfft_t<L>(const DevCurve *, int, const float2 *, \
                                                float2 *, const float4 *, const Plan &, \
                                                cudaStream_t);                       \
    template cudaError_t preload_pass1_t<3, L>();                                  \
    template cudaError_t preload_pass1_t<1, L>();                                  \
    template cudaError_t preload_pass2_t<L>(int);

}  // namespace cuvgls
