// Small complex DFTs and Cooley-Tukey butterflies in registers, shared by the
// shared-memory FFT kernels (fused z transform, one-pass 2D transforms).
#pragma once

namespace spme {

template <typename T>
struct Cx {
    T re, im;
};

template <typename T>
__device__ __forceinline__ Cx<T> cmul(Cx<T> a, Cx<T> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T>
__device__ __forceinline__ Cx<T> cadd(Cx<T> a, Cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T>
__device__ __forceinline__ Cx<T> csub(Cx<T> a, Cx<T> b) { return {a.re - b.re, a.im - b.im}; }

// cos and sin of 2 pi m / R for the radix-3 and radix-5 kernels
template <int R>
__device__ __forceinline__ double root_cos(int m);
template <int R>
__device__ __forceinline__ double root_sin(int m);
template <>
__device__ __forceinline__ double root_cos<3>(int m) { return m == 0 ? 1.0 : -0.5; }
template <>
__device__ __forceinline__ double root_sin<3>(int m) {
    return m == 0 ? 0.0 : (m == 1 ? 0.86602540378443865 : -0.86602540378443865);
}
// cos(2 pi/5) = (sqrt 5 - 1)/4, cos(4 pi/5) = -(sqrt 5 + 1)/4
template <>
__device__ __forceinline__ double root_cos<5>(int m) {
    return m == 0 ? 1.0 : ((m == 1 || m == 4) ? 0.30901699437494742 : -0.80901699437494742);
}
template <>
__device__ __forceinline__ double root_sin<5>(int m) {
    return m == 0 ? 0.0
                  : (m == 1 ? 0.95105651629515357
                            : (m == 2 ? 0.58778525229247313
                                      : (m == 3 ? -0.58778525229247313 : -0.95105651629515357)));
}

// Radix-R DFT of v into o: o[p] = sum_q v[q] w^{pq}, w = e^{-2 pi i/R}
// (forward) or its conjugate (INV).
template <typename T, int R, bool INV>
__device__ __forceinline__ void dft_small(const Cx<T> (&v)[R], Cx<T> (&o)[R]) {
    if constexpr (R == 1) {
        o[0] = v[0];
    } else if constexpr (R == 2) {
        o[0] = cadd(v[0], v[1]);
        o[1] = csub(v[0], v[1]);
    } else if constexpr (R == 4) {
        const Cx<T> s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        const Cx<T> s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
        // -i d13 forward, +i d13 inverse
        const Cx<T> jd = INV ? Cx<T>{-d13.im, d13.re} : Cx<T>{d13.im, -d13.re};
        o[0] = cadd(s02, s13);
        o[1] = cadd(d02, jd);
        o[2] = csub(s02, s13);
        o[3] = csub(d02, jd);
    } else {
#pragma unroll
        for (int p = 0; p < R; p++) {
            Cx<T> s = v[0];
#pragma unroll
            for (int q = 1; q < R; q++) {
                const int m = (p * q) % R;
                const T c = (T)root_cos<R>(m), sn = (T)(INV ? root_sin<R>(m) : -root_sin<R>(m));
                s.re += v[q].re * c - v[q].im * sn;
                s.im += v[q].re * sn + v[q].im * c;
            }
            o[p] = s;
        }
    }
}

// One radix-(R1 x R2) butterfly group of an in-place Cooley-Tukey pass with
// span L: v[q2][q1] = x[b L R1 R2 + j + q1 L + q2 L R1] (two consecutive radix
// stages, the R2 stage with span L R1).  Twiddles come from the KT-point table
// tw[e] = e^{-2 pi i e / KT} (KT a multiple of L R1 R2):
//   DIT (inverse):  t_q = x[j + q L] w^{q j};  x[j + p L] = sum_q t_q W_R^{pq}
//   DIF (forward):  x[j + q L] = (sum_p x[j + p L] W_R^{pq}) w^{q j}
// with w = e^{-2 pi i / (L R)} (conjugated, like W_R, for the inverse).  DIT
// runs the R1 stage first, DIF the R2 stage first; with L = 1 the R1 stage has
// no twiddles.
template <typename T, int R1, int R2, bool DIF, int L, int KT>
__device__ __forceinline__ void butterfly(Cx<T> (&v)[R2][R1], int j, const Cx<T> *__restrict__ tw) {
    constexpr int La = L * R1;
    constexpr int ts1 = KT / La, ts2 = KT / (La * R2);
    if constexpr (!DIF) {
#pragma unroll
        for (int q2 = 0; q2 < R2; q2++) {
            Cx<T> in[R1], out[R1];
#pragma unroll
            for (int q1 = 0; q1 < R1; q1++) in[q1] = v[q2][q1];
            if constexpr (L > 1) {
#pragma unroll
                for (int q1 = 1; q1 < R1; q1++) {
                    Cx<T> w = tw[q1 * j * ts1];
                    w.im = -w.im;
                    in[q1] = cmul(in[q1], w);
                }
            }
            dft_small<T, R1, true>(in, out);
#pragma unroll
            for (int p1 = 0; p1 < R1; p1++) v[q2][p1] = out[p1];
        }
        if constexpr (R2 > 1) {
#pragma unroll
            for (int p1 = 0; p1 < R1; p1++) {
                Cx<T> in[R2], out[R2];
                in[0] = v[0][p1];
#pragma unroll
                for (int q2 = 1; q2 < R2; q2++) {
                    Cx<T> w = tw[q2 * (j + p1 * L) * ts2];
                    w.im = -w.im;
                    in[q2] = cmul(v[q2][p1], w);
                }
                dft_small<T, R2, true>(in, out);
#pragma unroll
                for (int p2 = 0; p2 < R2; p2++) v[p2][p1] = out[p2];
            }
        }
    } else {
        if constexpr (R2 > 1) {
#pragma unroll
            for (int p1 = 0; p1 < R1; p1++) {
                Cx<T> in[R2], out[R2];
#pragma unroll
                for (int q2 = 0; q2 < R2; q2++) in[q2] = v[q2][p1];
                dft_small<T, R2, false>(in, out);
                v[0][p1] = out[0];
#pragma unroll
                for (int q2 = 1; q2 < R2; q2++) v[q2][p1] = cmul(out[q2], tw[q2 * (j + p1 * L) * ts2]);
            }
        }
#pragma unroll
        for (int q2 = 0; q2 < R2; q2++) {
            Cx<T> in[R1], out[R1];
#pragma unroll
            for (int p1 = 0; p1 < R1; p1++) in[p1] = v[q2][p1];
            dft_small<T, R1, false>(in, out);
            v[q2][0] = out[0];
#pragma unroll
            for (int q1 = 1; q1 < R1; q1++)
                v[q2][q1] = L > 1 ? cmul(out[q1], tw[q1 * j * ts1]) : out[q1];
        }
    }
}

}  // namespace spme
