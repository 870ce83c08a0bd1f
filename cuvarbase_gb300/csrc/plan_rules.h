// Compile-time rules shared by the host planner and the kernel templates:
// the menu of transform lengths, the radix sequence of each length, the
// tile shapes (columns B per pass-1 CTA, rows R per pass-2 CTA), the thread
// counts and the shared-memory footprints.  Host and device evaluate the
// same constexpr functions, so a plan the host picks always has a kernel.
#pragma once

#ifdef __CUDACC__
#define CUVGLS_HD __host__ __device__
#else
#define CUVGLS_HD
#endif

namespace cuvgls {

// Transform lengths with a compiled kernel: 2^a 5^c, multiples of 16.
constexpr int kLens[] = {16, 32, 64, 80, 128, 160, 256, 320, 400, 512,
                         640, 800, 1024, 1280, 1600, 2048};
constexpr int kNumLens = sizeof(kLens) / sizeof(kLens[0]);
// Row lengths (pass 2): the same and 4096.  A 4096-row grid (G up to
// 2048 x 4096) halves the sub-bands of very wide bands, and with them the
// spreading, which every sub-band repeats over all points of the curve; a
// 4096-long column tile would leave one column per pass-1 CTA and double the
// CTAs each record is spread into.
constexpr int kRowLens[] = {16, 32, 64, 80, 128, 160, 256, 320, 400, 512,
                            640, 800, 1024, 1280, 1600, 2048, 4096};
constexpr int kNumRowLens = sizeof(kRowLens) / sizeof(kRowLens[0]);

// Measured cost of the pass kernels on GB300, in ps per grid cell per curve,
// by transform length: pass 1 by column length G1 (kLens order), pass 2 by
// row length G2 (kRowLens order).  From 10,000-curve batches of curves with
// N log-uniform in [50, 5000] on 128,000- to 1,310,720-cell grids (ES window,
// m = 5); lengths marked * were not measured and are interpolated.  (The
// 320-long columns have since run 6 CTAs per SM instead of 5, 6 % faster;
// their entry is kept, since per cell pass 1 also depends on the points per
// curve and 6.1 would make 320 x 80 beat 160 x 160 at nf = 2e4, measured 8 %
// slower on these curves.)  Pass 1
// also pays per point (~0.23 ns per point of the curve, whatever the shape),
// which the shape choice can leave out.
constexpr float kPass1PsPerCell[] = {18.f /*16*/, 8.f /*32*/, 7.5f /*64 **/, 8.6f /*80*/,
                                     7.f /*128 **/, 6.4f /*160*/, 7.1f /*256*/, 6.5f /*320*/,
                                     6.3f /*400*/, 6.8f /*512*/, 6.f /*640*/, 6.8f /*800*/,
                                     6.5f /*1024*/, 15.2f /*1280*/, 20.5f /*1600*/,
                                     22.f /*2048 **/};
constexpr float kPass2PsPerCell[] = {6.7f /*16*/, 6.2f /*32*/, 8.5f /*64*/, 7.9f /*80*/,
                                     8.5f /*128 **/, 7.9f /*160*/, 9.3f /*256*/, 9.3f /*320*/,
                                     7.f /*400*/, 9.9f /*512*/, 8.4f /*640*/, 9.6f /*800*/,
                                     12.f /*1024*/, 20.f /*1280*/, 25.5f /*1600*/,
                                     28.f /*2048 **/, 30.f /*4096 **/};
static_assert(sizeof(kPass1PsPerCell) / sizeof(float) == sizeof(kLens) / sizeof(int),
              "one pass-1 cost per column length");
static_assert(sizeof(kPass2PsPerCell) / sizeof(float) == sizeof(kRowLens) / sizeof(int),
              "one pass-2 cost per row length");

// Elements a thread holds in registers during one FFT stage (target).
constexpr int kEPT = 16;
constexpr int kMaxThreads = 1024;
constexpr int kMaxTile = kEPT * kMaxThreads;  // complex elements per CTA
constexpr int kSmemLimit = 227 * 1024;
constexpr int kMaxFac = 12;

struct FacList {
    int n;
    int r[kMaxFac];
};

// Radix sequence of L = 2^a 5^c: the radix-5 stages first, then 16s, then
// the remaining power of two (2, 4, 8 or 16).
CUVGLS_HD constexpr FacList fft_factors(int L) {
    FacList f{0, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
    int x = L;
    while (x % 5 == 0) { f.r[f.n++] = 5; x /= 5; }
    while (x % 3 == 0) { f.r[f.n++] = 3; x /= 3; }
    while (x % 16 == 0 && x > 16) { f.r[f.n++] = 16; x /= 16; }
    if (x > 1) f.r[f.n++] = x;
    return f;
}

CUVGLS_HD constexpr bool len_ok(int L) {
    FacList f = fft_factors(L);
    int p = 1;
    for (int i = 0; i < f.n; ++i) {
        int r = f.r[i];
        if (r != 2 && r != 3 && r != 4 && r != 5 && r != 8 && r != 16) return false;
        p *= r;
    }
    return p == L;
}

// Product of the radices before stage s (the Stockham span Ns).
CUVGLS_HD constexpr int fft_ns(int L, int s) {
    FacList f = fft_factors(L);
    int p = 1;
    for (int i = 0; i < s; ++i) p *= f.r[i];
    return p;
}

// Stage twiddles are stored per stage as [r = 1..R-1][k = 0..Ns-1]; stage 0
// (Ns = 1) needs none.  Offset of stage s and the total table length.
CUVGLS_HD constexpr int stage_tw_offset(int L, int s) {
    FacList f = fft_factors(L);
    int off = 0, ns = 1;
    for (int i = 0; i < s; ++i) {
        if (ns > 1) off += ns * (f.r[i] - 1);
        ns *= f.r[i];
    }
    return off;
}
CUVGLS_HD constexpr int stage_tw_total(int L) {
    return stage_tw_offset(L, fft_factors(L).n);
}

// Padded position of element i along a transform: one slot after every 16
// elements, which spreads the strided Stockham writes over the banks.
CUVGLS_HD constexpr int padded(int i) { return i + (i >> 4); }
CUVGLS_HD constexpr int padded_len(int L) { return L + (L >> 4); }

// Two-level split L = La * Lb with both factors register-DFT sizes (<= 32);
// La is the factor closest to sqrt(L) from below, unless that leaves Lb not
// a multiple of 4: then the split with Lb a multiple of 4 and La closest to
// sqrt(L) (so that a pass-2 stage A can read whole 4-column blocks; this
// only changes 80 = 10 x 8).  0 when there is none.
CUVGLS_HD constexpr bool reg_dft_ok(int r) {
    return r == 4 || r == 5 || r == 8 || r == 10 || r == 16 || r == 20 || r == 25 ||
           r == 32;
}
CUVGLS_HD constexpr int two_level_la(int L) {
    int best = 0;
    for (int la = 4; la <= 32; ++la)
        if (L % la == 0 && reg_dft_ok(la) && reg_dft_ok(L / la) && la * la <= L) best = la;
    if (best == 0 || (L / best) % 4 == 0) return best;
    int alt = 0;
    long long dist = 0;
    for (int la = 4; la <= 32; ++la)
        if (L % la == 0 && reg_dft_ok(la) && reg_dft_ok(L / la) && (L / la) % 4 == 0) {
            const long long d = (long long)la * la > L ? (long long)la * la - L
                                                       : L - (long long)la * la;
            if (alt == 0 || d < dist) { alt = la; dist = d; }
        }
    return alt ? alt : best;
}

// Position of element n of a length-L tile vector: two-level lengths pad one
// slot per Lb elements, the others one per 16.
CUVGLS_HD constexpr int phys2_len(int L) {
    return two_level_la(L) ? L + L / (L / two_level_la(L)) : padded_len(L);
}

CUVGLS_HD constexpr int threads_for(int elems) {
    return elems <= kEPT * 128 ? 128
         : elems <= kEPT * 256 ? 256
         : elems <= kEPT * 512 ? 512 : 1024;
}

template <int L>
CUVGLS_HD constexpr int phys2(int n) {
    if constexpr (two_level_la(L) > 0) {
        constexpr int LB = L / two_level_la(L);
        return n + n / LB;
    } else {
        return padded(n);
    }
}

// Table an FFT of length L reads: the [qa][i] stage-A twiddles of a
// two-level length, the Stockham stage twiddles otherwise.
CUVGLS_HD constexpr int fft_table_len(int L) {
    return two_level_la(L) ? L : stage_tw_total(L);
}
CUVGLS_HD constexpr int tile_len(int L) { return phys2_len(L); }
// Row stride of a pass-2 tile.
CUVGLS_HD constexpr int row_stride(int L) { return tile_len(L); }
CUVGLS_HD constexpr int round32(int x) { return (x + 31) / 32 * 32; }

// Threads for V vectors of length L: one per stage-B unit of a two-level
// length (at least 128), the Stockham rule otherwise.
CUVGLS_HD constexpr int fft_threads(int V, int L) {
    return two_level_la(L) ? (round32(V * two_level_la(L)) < 128 ? 128
                                                                   : round32(V * two_level_la(L)))
                           : threads_for(V * L);
}
CUVGLS_HD constexpr bool tile_fits(int V, int L) {
    return two_level_la(L) ? V * two_level_la(L) <= kMaxThreads : V * L <= kMaxTile;
}

// Columns per pass-1 CTA for ng grids of column length L1.
CUVGLS_HD constexpr int pass1_cols(int ng, int L1) {
    int b = (ng == 1) ? 8 : 4;
    while (b > 2 && !tile_fits(ng * b, L1)) b /= 2;
    return b;
}

// Rows per pass-2 CTA for ng grids of row length L2: 16 for short rows, so
// that a CTA still transforms a few thousand elements; 4 for the three-grid
// GLS rows of 256..1024 (more, smaller CTAs per SM overlap one CTA's loads
// with another's arithmetic); 8 otherwise; halved until the tile fits (2 at
// least, 1 only for the 4096-long rows).
CUVGLS_HD constexpr int pass2_rows(int ng, int L2) {
    int r = (ng == 1 || L2 <= 160) ? 16 : (L2 <= 1024 ? 4 : 8);
    while (r > (L2 > 2048 ? 1 : 2) && !tile_fits(ng * r, L2)) r /= 2;
    return r;
}

CUVGLS_HD constexpr int pass1_threads(int ng, int L1) {
    return fft_threads(ng * pass1_cols(ng, L1), L1);
}
CUVGLS_HD constexpr int pass2_threads(int ng, int L2) {
    return fft_threads(ng * pass2_rows(ng, L2), L2);
}

// Shared memory (bytes) of a pass-1 CTA: ng padded column tiles (and the
// Stockham twiddles for lengths without a two-level split), then the staged
// records (packed row/column, offset, two complex values; 24 bytes each).
constexpr int kStageRecBytes = 24;

CUVGLS_HD constexpr long long pass1_tile_bytes(int ng, int L1) {
    // two-level lengths read their FFT table through the read-only cache;
    // Stockham lengths stage it in shared memory
    return (long long)(ng * tile_len(L1) * pass1_cols(ng, L1) +
                       (two_level_la(L1) ? 0 : fft_table_len(L1))) * 8;
}

// Records a pass-1 CTA stages per round: 256, or, for the 1024-thread CTAs
// of the long Stockham columns (one CTA per SM), as many as fit (in steps of
// 256, up to 4096) beside the row counts and the row-sorted record list of
// the gather spreading, so that a dense curve (tens of thousands of records
// per column block) takes a few rounds rather than one barrier pair per 256
// records.
CUVGLS_HD constexpr bool pass1_gather(int ng, int L1) { return pass1_threads(ng, L1) == 1024; }

// Gather spreading's extra shared memory: L1 + 1 row counts, one record
// index per staged record, 32 warp sums of the block scan.
CUVGLS_HD constexpr long long pass1_gather_bytes(int L1, int recs) {
    return (long long)(L1 + 1 + recs + 32) * 4;
}

// Row-residue occupancy flags of the sparse spreading: one byte per (record
// kind, residue i < Lb) of the two-level column FFT, which lets stage A skip
// the all-zero units.
constexpr int kOccBytes = 64;

// CTAs per SM that `bytes` of shared memory per CTA allow (228 KB per SM,
// 1 KB of it reserved per CTA).
CUVGLS_HD constexpr int smem_ctas(long long bytes) { return (int)(233472 / (bytes + 1024)); }

// Registers a thread of the pass-1 kernels needs without spilling (56-60
// across the lengths).
constexpr int kPass1Regs = 56;

// Whether staging 192 records per round instead of 256 fits one more pass-1
// CTA per SM of the three GLS grids, within the register budget of
// kPass1Regs per thread: on the 320-long columns (192 threads) 6 CTAs per SM
// instead of 5, pass 1 of the bench workload 9.62 -> 9.08 ms.  (Only the
// three-grid tiles, where it was measured; the one-grid NFFT tiles keep 256.)
CUVGLS_HD constexpr bool pass1_small_stage(int ng, int L1) {
    return ng == 3 && !pass1_gather(ng, L1) &&
           smem_ctas(pass1_tile_bytes(ng, L1) + kOccBytes + 192LL * kStageRecBytes) >
               smem_ctas(pass1_tile_bytes(ng, L1) + kOccBytes + 256LL * kStageRecBytes) &&
           65536 / (pass1_threads(ng, L1) *
                    smem_ctas(pass1_tile_bytes(ng, L1) + kOccBytes + 192LL * kStageRecBytes)) >=
               kPass1Regs;
}

// CTAs per SM a pass-1 kernel is compiled to keep resident (its launch
// bound): the small-stage count, else 1 (no register cap).
CUVGLS_HD constexpr int pass1_min_ctas(int ng, int L1) {
    return pass1_small_stage(ng, L1)
               ? smem_ctas(pass1_tile_bytes(ng, L1) + kOccBytes + 192LL * kStageRecBytes)
               : 1;
}

CUVGLS_HD constexpr int pass1_stage_recs(int ng, int L1) {
    if (!pass1_gather(ng, L1)) return pass1_small_stage(ng, L1) ? 192 : 256;
    int r = 4096;
    while (r > 256 && pass1_tile_bytes(ng, L1) + (long long)r * kStageRecBytes +
                              pass1_gather_bytes(L1, r) + kOccBytes > kSmemLimit)
        r -= 256;
    return r;
}

CUVGLS_HD constexpr long long pass1_smem(int ng, int L1, long long G) {
    return pass1_tile_bytes(ng, L1) + (long long)pass1_stage_recs(ng, L1) * kStageRecBytes +
           (pass1_gather(ng, L1) ? pass1_gather_bytes(L1, pass1_stage_recs(ng, L1)) : 0) +
           kOccBytes;
}

// Shared memory of a pass-2 CTA: ng * R padded rows and the stage twiddles.
CUVGLS_HD constexpr long long pass2_smem(int ng, int L2) {
    return (long long)(ng * pass2_rows(ng, L2) * row_stride(L2) +
                       (two_level_la(L2) ? 0 : fft_table_len(L2))) * 8;
}

}  // namespace cuvgls
