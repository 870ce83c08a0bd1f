// In-place mixed-radix Stockham FFTs (inverse sign, unnormalised) on tiles in
// shared memory.  One CTA transforms `nvec` vectors of length L at once.
//
// Stage s with radix R and Ns = product of the earlier radices: butterfly j
// (0 <= j < L/R) reads elements j + r L/R, multiplies element r by
// exp(+2 pi i (j mod Ns) r / (Ns R)), does an R-point DFT and writes element
// r to (j / Ns) Ns R + (j mod Ns) + r Ns.  The output comes out in natural
// order (Stockham autosort).  Each stage reads all of its butterflies into
// registers, synchronises, then writes, so the tile is transformed in place.
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

// Vector v of the tile starts at (v % vin) * s_in + (v / vin) * s_out and its
// elements are es apart.
struct TileLayout {
    int nvec, vin, s_in, s_out, es;
};

template <int R, int IT>
__device__ __forceinline__ void stockham_stage(float2 *__restrict__ buf, int L,
                                               int Ns, TileLayout lay,
                                               const float2 *__restrict__ tw,
                                               int nthr, int tid) {
    const int nb = L / R;
    const int tot = lay.nvec * nb;
    const int tstep = L / (Ns * R);
    // Zero-initialised so that no value is live on the paths that skip a
    // butterfly; without it the compiler keeps every radix case's arrays
    // alive at once.
    float2 v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[it][r] = make_float2(0.f, 0.f);
        const int bf = tid + it * nthr;
        if (bf < tot) {
            const int c = bf % lay.vin;
            const int rest = bf / lay.vin;
            const int j = rest % nb;
            const int vo = rest / nb;
            const int base = c * lay.s_in + vo * lay.s_out;
            const int k = j % Ns;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                float2 a = buf[base + (j + r * nb) * lay.es];
                if (r > 0) a = cmul(a, tw[k * r * tstep]);
                v[it][r] = a;
            }
            SmallDFT<R>::run(v[it]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int bf = tid + it * nthr;
        if (bf < tot) {
            const int c = bf % lay.vin;
            const int rest = bf / lay.vin;
            const int j = rest % nb;
            const int vo = rest / nb;
            const int base = c * lay.s_in + vo * lay.s_out;
            const int k = j % Ns;
            const int d = (j / Ns) * Ns * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) buf[base + (d + r * Ns) * lay.es] = v[it][r];
        }
    }
    __syncthreads();
}

// Full transform of every vector of the tile.  Requires
// lay.nvec * L <= kEPT * nthr.  tw = exp(+2 pi i n / L), n < L.  fac holds
// the radices, 5 bits each, first stage in the lowest bits.
__device__ __forceinline__ void smem_fft(float2 *__restrict__ buf, int L,
                                         unsigned long long fac, int nfac,
                                         TileLayout lay,
                                         const float2 *__restrict__ tw, int nthr,
                                         int tid) {
    int Ns = 1;
    for (int s = 0; s < nfac; ++s) {
        const int R = (int)((fac >> (5 * s)) & 31u);
        switch (R) {
        case 2: stockham_stage<2, (kEPT + 1) / 2>(buf, L, Ns, lay, tw, nthr, tid); break;
        case 3: stockham_stage<3, (kEPT + 2) / 3>(buf, L, Ns, lay, tw, nthr, tid); break;
        case 4: stockham_stage<4, (kEPT + 3) / 4>(buf, L, Ns, lay, tw, nthr, tid); break;
        case 5: stockham_stage<5, (kEPT + 4) / 5>(buf, L, Ns, lay, tw, nthr, tid); break;
        case 8: stockham_stage<8, (kEPT + 7) / 8>(buf, L, Ns, lay, tw, nthr, tid); break;
        default: stockham_stage<16, (kEPT + 15) / 16>(buf, L, Ns, lay, tw, nthr, tid); break;
        }
        Ns *= R;
    }
}

}  // namespace cuvgls
