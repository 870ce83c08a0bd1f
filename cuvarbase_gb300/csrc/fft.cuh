// In-place mixed-radix Stockham FFTs (inverse sign, unnormalised) on tiles in
// shared memory.  One CTA transforms V vectors of a compile-time length L.
//
// Stage s with radix R and span Ns (product of the earlier radices):
// butterfly j (0 <= j < L/R) reads elements j + r L/R, multiplies element r
// by exp(+2 pi i (j mod Ns) r / (Ns R)), runs an R-point DFT and writes
// element r to (j / Ns) Ns R + (j mod Ns) + r Ns.  The output is in natural
// order.  Each stage reads all of its butterflies into registers,
// synchronises, then writes, so the tile is transformed in place.
//
// Everything that shapes the index arithmetic (L, R, Ns, the tile layout and
// the thread count) is a template parameter, so divisions and remainders are
// by constants.  Element i of vector v lives at
//   base(v) + padded(i) * ES,  base(v) = (v % VIN) * SIN + (v / VIN) * SOUT,
// padded(i) = i + i / 16 (one spare slot per 16 elements keeps the strided
// stores of the early stages off a single bank).
#pragma once

#include "common.cuh"

namespace cuvgls {

template <int R> struct SmallDFT;

template <> struct SmallDFT<2> {
    static __device__ __forceinline__ void run(float2 *v) {
        float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <> struct SmallDFT<3> {
    static __device__ __forceinline__ void run(float2 *v) {
        const float h = 0.86602540378443864676f;  // sin(2 pi / 3)
        float2 s = cadd(v[1], v[2]);
        float2 d = cmuli(cscale(csub(v[1], v[2]), h));
        float2 m = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
        v[0] = cadd(v[0], s);
        v[1] = cadd(m, d);
        v[2] = csub(m, d);
    }
};

template <> struct SmallDFT<4> {
    static __device__ __forceinline__ void run(float2 *v) {
        float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        float2 t2 = cadd(v[1], v[3]), t3 = cmuli(csub(v[1], v[3]));
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    }
};

template <> struct SmallDFT<5> {
    static __device__ __forceinline__ void run(float2 *v) {
        const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
        const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
        const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
        const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
        float2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
        float2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
        float2 m1 = make_float2(v[0].x + c1 * a1.x + c2 * a2.x,
                                v[0].y + c1 * a1.y + c2 * a2.y);
        float2 m2 = make_float2(v[0].x + c2 * a1.x + c1 * a2.x,
                                v[0].y + c2 * a1.y + c1 * a2.y);
        float2 n1 = cmuli(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
        float2 n2 = cmuli(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
        v[0] = cadd(v[0], cadd(a1, a2));
        v[1] = cadd(m1, n1);
        v[4] = csub(m1, n1);
        v[2] = cadd(m2, n2);
        v[3] = csub(m2, n2);
    }
};

// Radix 8 = two radix-4 DFTs of the even / odd elements plus one radix-2 layer.
template <> struct SmallDFT<8> {
    static __device__ __forceinline__ void run(float2 *v) {
        const float r = 0.70710678118654752440f;
        float2 e[4] = {v[0], v[2], v[4], v[6]};
        float2 o[4] = {v[1], v[3], v[5], v[7]};
        SmallDFT<4>::run(e);
        SmallDFT<4>::run(o);
        // exp(+2 pi i k / 8), k = 0..3
        float2 w1 = cmul(o[1], make_float2(r, r));
        float2 w2 = cmuli(o[2]);
        float2 w3 = cmul(o[3], make_float2(-r, r));
        v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], w1);   v[5] = csub(e[1], w1);
        v[2] = cadd(e[2], w2);   v[6] = csub(e[2], w2);
        v[3] = cadd(e[3], w3);   v[7] = csub(e[3], w3);
    }
};

// Radix 16 = two radix-8 DFTs plus one radix-2 layer.
template <> struct SmallDFT<16> {
    static __device__ __forceinline__ void run(float2 *v) {
        const float c8 = 0.92387953251128675613f;  // cos(pi / 8)
        const float s8 = 0.38268343236508977173f;  // sin(pi / 8)
        const float r = 0.70710678118654752440f;
        float2 e[8], o[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
        SmallDFT<8>::run(e);
        SmallDFT<8>::run(o);
        const float2 w[8] = {make_float2(1.f, 0.f), make_float2(c8, s8),
                             make_float2(r, r),     make_float2(s8, c8),
                             make_float2(0.f, 1.f), make_float2(-s8, c8),
                             make_float2(-r, r),    make_float2(-c8, s8)};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float2 t = (k == 0) ? o[0] : cmul(o[k], w[k]);
            v[k] = cadd(e[k], t);
            v[k + 8] = csub(e[k], t);
        }
    }
};

// One Stockham stage.  tws holds the stage twiddles of L as
// [stage][r - 1][k] (see stage_tw_offset).
template <int L, int S, int V, int VIN, int SIN, int SOUT, int ES, int NT>
struct FftStage {
    static constexpr int R = fft_factors(L).r[S];
    static constexpr int NS = fft_ns(L, S);
    static constexpr int NB = L / R;
    static constexpr int TOT = V * NB;
    static constexpr int IT = (TOT + NT - 1) / NT;
    static constexpr int TWO = stage_tw_offset(L, S);

    static __device__ __forceinline__ void run(float2 *__restrict__ buf,
                                               const float2 *__restrict__ tws,
                                               int tid) {
        // Zero-initialised so that no value is live on the paths that skip a
        // butterfly (keeps the register allocation per stage).
        float2 v[IT][R];
#pragma unroll
        for (int it = 0; it < IT; ++it) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[it][r] = make_float2(0.f, 0.f);
            const int bf = tid + it * NT;
            if (TOT % NT == 0 || bf < TOT) {
                const int c = bf % VIN;
                const int rest = bf / VIN;
                const int j = rest % NB;
                const int vo = rest / NB;
                const int base = c * SIN + vo * SOUT;
                const int k = j % NS;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    float2 a = buf[base + padded(j + r * NB) * ES];
                    if (NS > 1 && r > 0) a = cmul(a, tws[TWO + (r - 1) * NS + k]);
                    v[it][r] = a;
                }
                SmallDFT<R>::run(v[it]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < IT; ++it) {
            const int bf = tid + it * NT;
            if (TOT % NT == 0 || bf < TOT) {
                const int c = bf % VIN;
                const int rest = bf / VIN;
                const int j = rest % NB;
                const int vo = rest / NB;
                const int base = c * SIN + vo * SOUT;
                const int d = (j / NS) * NS * R + j % NS;
#pragma unroll
                for (int r = 0; r < R; ++r) buf[base + padded(d + r * NS) * ES] = v[it][r];
            }
        }
        __syncthreads();
    }
};

template <int L, int S, int V, int VIN, int SIN, int SOUT, int ES, int NT>
__device__ __forceinline__ void fft_stages(float2 *__restrict__ buf,
                                           const float2 *__restrict__ tws, int tid) {
    if constexpr (S < fft_factors(L).n) {
        FftStage<L, S, V, VIN, SIN, SOUT, ES, NT>::run(buf, tws, tid);
        fft_stages<L, S + 1, V, VIN, SIN, SOUT, ES, NT>(buf, tws, tid);
    }
}

// Transform every vector of the tile (see the layout above).
template <int L, int V, int VIN, int SIN, int SOUT, int ES, int NT>
__device__ __forceinline__ void tile_fft(float2 *__restrict__ buf,
                                         const float2 *__restrict__ tws, int tid) {
    static_assert(len_ok(L), "length must be 2^a 3^b 5^c with supported radices");
    fft_stages<L, 0, V, VIN, SIN, SOUT, ES, NT>(buf, tws, tid);
}


// ===========================================================================
// Two-level ("four-step") tile FFT for L = La * Lb with La, Lb <= 32.
//
// Element n = i + Lb k (i < Lb, k < La) is stored at phys(n) = n + n / Lb (one
// spare slot per Lb elements).  Output q = qa + La qb.
//   stage A, per (vector, i):  Y[qa] = W_L^(i qa) * sum_k x[i + Lb k] W_La^(k qa),
//            stored in place at i + Lb qa (a thread owns its column: no sync
//            between its reads and writes);
//   stage B, per (vector, qa): X[qa + La qb] = sum_i Y_i[qa] W_Lb^(i qb),
//            read from the contiguous block Lb qa .. Lb qa + Lb - 1.
// Both DFTs run in registers with compile-time twiddles.  The stage-A
// twiddles W_L^(i qa) come from a [qa][i] table (consecutive threads read
// consecutive entries).  With the padding, the strided reads of stage B
// (stride Lb + 1, odd) and all other accesses are free of bank conflicts.
// ===========================================================================

// Compile-time cos / sin of 2 pi a / b (Taylor series on |x| <= pi).
constexpr double kPiC = 3.14159265358979323846264338327950288;
constexpr double taylor_sin(double x) {
    double term = x, sum = x;
    for (int n = 1; n < 16; ++n) { term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0)); sum += term; }
    return sum;
}
constexpr double taylor_cos(double x) {
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 16; ++n) { term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n)); sum += term; }
    return sum;
}
constexpr double turn_angle(int a, int b) {
    int r = a % b;
    if (r < 0) r += b;
    if (2 * r > b) r -= b;
    return 2.0 * kPiC * (double)r / (double)b;
}
constexpr float cos_turn(int a, int b) { return (float)taylor_cos(turn_angle(a, b)); }
constexpr float sin_turn(int a, int b) { return (float)taylor_sin(turn_angle(a, b)); }

template <int R> struct RegDFT;

template <int P, int Q, int N2, int K1>
__device__ __forceinline__ float2 comp_twiddle(float2 a) {
    constexpr int e = (N2 * K1) % (P * Q);
    if constexpr (e == 0) {
        return a;
    } else {
        constexpr float c = cos_turn(e, P * Q);
        constexpr float s = sin_turn(e, P * Q);
        return cmul(a, make_float2(c, s));
    }
}

// step 1 of a composite DFT: for column N2, a P-point DFT, then twiddles
template <int P, int Q, int N2, int K1>
struct CompTw {
    static __device__ __forceinline__ void run(const float2 *t, float2 *y) {
        if constexpr (K1 < P) {
            y[N2 * P + K1] = comp_twiddle<P, Q, N2, K1>(t[K1]);
            CompTw<P, Q, N2, K1 + 1>::run(t, y);
        }
    }
};

template <int P, int Q, int N2>
struct CompStep1 {
    static __device__ __forceinline__ void run(const float2 *v, float2 *y) {
        if constexpr (N2 < Q) {
            float2 t[P];
#pragma unroll
            for (int n1 = 0; n1 < P; ++n1) t[n1] = v[Q * n1 + N2];
            RegDFT<P>::run(t);
            CompTw<P, Q, N2, 0>::run(t, y);
            CompStep1<P, Q, N2 + 1>::run(v, y);
        }
    }
};

// R = P Q point inverse DFT in registers: n = Q n1 + n2, k = k1 + P k2.
template <int P, int Q>
struct CompositeDFT {
    static __device__ __forceinline__ void run(float2 *v) {
        float2 y[P * Q];
        CompStep1<P, Q, 0>::run(v, y);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
            float2 t[Q];
#pragma unroll
            for (int n2 = 0; n2 < Q; ++n2) t[n2] = y[n2 * P + k1];
            RegDFT<Q>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < Q; ++k2) v[k1 + P * k2] = t[k2];
        }
    }
};

template <int R> struct RegDFT : SmallDFT<R> {};
template <> struct RegDFT<10> : CompositeDFT<2, 5> {};
template <> struct RegDFT<20> : CompositeDFT<4, 5> {};
template <> struct RegDFT<25> : CompositeDFT<5, 5> {};
template <> struct RegDFT<32> : CompositeDFT<4, 8> {};

// Two-level FFT of length L = LA LB (LA = two_level_la(L)).  Element
// n = i + LB k (i < LB, k < LA).  Stage A, one unit per (vector, i): a
// length-LA DFT over k, then the twiddle exp(2 pi i qa i / L), leaving
// intermediate i + LB qa.  Stage B, one unit per (vector, qa): a length-LB
// DFT over i, giving output q = qa + LA qb.

// Padded position of element i + LB k of a two-level length, 0 <= i < LB
// (equal to phys2<L>(i + LB k), without its division).
template <int L>
__device__ __forceinline__ constexpr int phys2_ik(int i, int k) {
    return i + (L / two_level_la(L) + 1) * k;
}

// Stage A of one unit in registers: x[k] = element i + LB k on entry,
// x[qa] = intermediate i + LB qa on return.
template <int L>
__device__ __forceinline__ void fft2_stage_a_regs(float2 (&x)[two_level_la(L)],
                                                  const float2 *__restrict__ twa, int i) {
    constexpr int LA = two_level_la(L);
    constexpr int LB = L / LA;
    RegDFT<LA>::run(x);
#pragma unroll
    for (int qa = 1; qa < LA; ++qa) x[qa] = cmul(x[qa], __ldg(twa + qa * LB + i));
}

// Stage A over every vector of a tile, in place (no barrier at the end).
template <int L, int V, int VIN, int SIN, int SOUT, int ES, int NT>
__device__ __forceinline__ void tile_fft2_a(float2 *__restrict__ buf,
                                            const float2 *__restrict__ twa, int tid) {
    constexpr int LA = two_level_la(L);
    constexpr int LB = L / LA;
    static_assert(LA > 0, "length has no two-level split");
#pragma unroll 1
    for (int u = tid; u < V * LB; u += NT) {
        const int c = u % VIN;
        const int rest = u / VIN;
        const int i = rest % LB;
        const int vo = rest / LB;
        const int base = c * SIN + vo * SOUT;
        float2 x[LA];
#pragma unroll
        for (int k = 0; k < LA; ++k) x[k] = buf[base + phys2_ik<L>(i, k) * ES];
        fft2_stage_a_regs<L>(x, twa, i);
#pragma unroll
        for (int qa = 0; qa < LA; ++qa) buf[base + phys2_ik<L>(i, qa) * ES] = x[qa];
    }
}

// Stage B of the unit of this thread (at most one: NT >= V LA): reads the
// LB intermediates of (vector, qa) and transforms them; y[qb] is output
// qa + LA qb of vector (vo, c).  Returns false for threads without a unit.
template <int L, int V, int VIN, int SIN, int SOUT, int ES, int NT>
__device__ __forceinline__ bool tile_fft2_b(const float2 *__restrict__ buf, int tid,
                                            float2 (&y)[L / two_level_la(L)], int &vo,
                                            int &c, int &qa) {
    constexpr int LA = two_level_la(L);
    constexpr int LB = L / LA;
    static_assert(NT >= V * LA, "stage B needs one thread per unit");
    if (tid >= V * LA) return false;
    c = tid % VIN;
    const int rest = tid / VIN;
    qa = rest % LA;
    vo = rest / LA;
    const int base = c * SIN + vo * SOUT;
#pragma unroll
    for (int i = 0; i < LB; ++i) y[i] = buf[base + phys2_ik<L>(i, qa) * ES];
    RegDFT<LB>::run(y);
    return true;
}

// Stage B in place: output q of each vector at its natural position.
template <int L, int V, int VIN, int SIN, int SOUT, int ES, int NT>
__device__ __forceinline__ void tile_fft2_b_inplace(float2 *__restrict__ buf, int tid) {
    constexpr int LA = two_level_la(L);
    constexpr int LB = L / LA;
    float2 y[LB];
    int vo = 0, c = 0, qa = 0;
    const bool act = tile_fft2_b<L, V, VIN, SIN, SOUT, ES, NT>(buf, tid, y, vo, c, qa);
    __syncthreads();
    if (act) {
        const int base = c * SIN + vo * SOUT;
#pragma unroll
        for (int qb = 0; qb < LB; ++qb) {
            // qa + LA qb; with LA == LB, qa < LB is the in-row index
            const int o = (LA == LB) ? phys2_ik<L>(qa, qb) : phys2<L>(qa + LA * qb);
            buf[base + o * ES] = y[qb];
        }
    }
    __syncthreads();
}

template <int L, int V, int VIN, int SIN, int SOUT, int ES, int NT>
__device__ __forceinline__ void tile_fft2(float2 *__restrict__ buf,
                                          const float2 *__restrict__ twa, int tid) {
    tile_fft2_a<L, V, VIN, SIN, SOUT, ES, NT>(buf, twa, tid);
    __syncthreads();
    tile_fft2_b_inplace<L, V, VIN, SIN, SOUT, ES, NT>(buf, tid);
}

// Transform every vector of a tile with the two-level FFT when L has a
// split, the Stockham FFT otherwise; `tab` is fft_table_len(L) entries.
template <int L, int V, int VIN, int SIN, int SOUT, int ES, int NT>
__device__ __forceinline__ void tile_fft_any(float2 *__restrict__ buf,
                                             const float2 *__restrict__ tab, int tid) {
    if constexpr (two_level_la(L) > 0) tile_fft2<L, V, VIN, SIN, SOUT, ES, NT>(buf, tab, tid);
    else tile_fft<L, V, VIN, SIN, SOUT, ES, NT>(buf, tab, tid);
}

}  // namespace cuvgls
