// GLS power from the trigonometric sums of one frequency (shared by the
// NFFT finish and the direct-sum kernel).
#pragma once

#include <cuda_runtime.h>

namespace cuvgls {

// 2x2 normal equations of the sinusoid fit; P = b^T A^-1 b * pnorm.
// mode 1 (floating mean): cuvarbase/lombscargle.py:337-536 (H=1) and
// cuvarbase/kernels/lomb.cu:36-83; mode 0 (standard): lomb.cu:85-123;
// mode 2 (window): lomb.cu:136-137.  The closed forms in lomb.cu rotate to
// the frame where A is diagonal; the value is the same.  Invalid -> -1.
template <typename T>
__device__ __forceinline__ T gls_from_sums(T YCh, T YSh, T C, T S, T C2, T S2,
                                           int mode, T reg, T wsum, T ywsum,
                                           T ybar, T pnorm) {
    T YC, YS, CC, SS, CS;
    const T half = (T)0.5;
    if (mode == 1) {
        YC = YCh - ywsum * C;
        YS = YSh - ywsum * S;
        CC = half * (wsum + C2) - C * C + reg;
        SS = half * (wsum - C2) - S * S + reg;
        CS = half * S2 - C * S;
    } else if (mode == 0) {
        YC = YCh + ybar * C;
        YS = YSh + ybar * S;
        CC = half * ((T)1 + C2) + reg;
        SS = half * ((T)1 - C2) + reg;
        CS = half * S2;
    } else {
        YC = C + C;
        YS = S + S;
        CC = half * ((T)1 + C2);
        SS = half * ((T)1 - C2);
        CS = half * S2;
    }
    const T det = CC * SS - CS * CS;
    const T num = YC * YC * SS - (T)2 * YC * YS * CS + YS * YS * CC;
    T P;
    if constexpr (sizeof(T) == 4) P = __fdividef(num, det) * pnorm;
    else P = num / det * pnorm;
    if (!(P >= (T)0) || isinf(P)) P = (T)-1;
    return P;
}

}  // namespace cuvgls
