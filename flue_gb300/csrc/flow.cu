// flow.cu -- Luescher's Wilson flow (M. Luescher, JHEP 08 (2010) 071,
// appendix C) with the 3-stage Runge-Kutta integrator, in place on a device
// field.  No reference counterpart.
//
// Flow velocity: dV/dt = Z(V) V with Z = -g0^2 d S_w summed over oriented
// plaquettes, i.e. Z = 2 G where G = -1/2 TA(U N) is the su(3) gradient of
// sum_{x,mu<nu} Re Tr P (k_plaqforce in force.cu, Lie form).  One step with
// the low-storage form of the integrator:
//     Z0 = eps Z(W0);  W1 = exp(Z0/4) W0;                 B = Z0
//     Z1 = eps Z(W1);  X = 8/9 Z1 - 17/36 B; W2 = exp(X) W1; B = X
//     Z2 = eps Z(W2);  W3 = exp(3/4 Z2 - B) W2
// The update runs in the field's precision: D = exp(X) - I by the Taylor
// series summed in the basis {I, X, X^2} (expm1_m3 below), scaled and squared
// for |X| > 1/2 (Moler & Van Loan, "Nineteen dubious ways to compute the
// exponential of a matrix", methods 3 and 8), then W' = W + D W.  Keeping the
// small D apart from I holds its relative precision in FP32, so the update
// adds one rounding of W per stage, as an FP64 update rounded to FP32 would.
// FP32 fields are reunitarised (FixSU3Matrix) after every stage.
#include "flue_internal.h"

namespace flue {

size_t wflow_ws_bytes(const Geom& g) {
    // force (4 x 9 complex doubles per site), B (4 x 9 reals per site),
    // plaquette partials
    const size_t f = (size_t)36 * g.V * 16;
    const size_t b = (size_t)36 * g.V * 8;
    const size_t p = (size_t)plaqforce_blocks(g) * 4 * 8;
    return ((f + 255) & ~(size_t)255) + ((b + 255) & ~(size_t)255) + ((p + 255) & ~(size_t)255);
}

template <typename T>
struct Cx {
    T re, im;
};
template <typename T>
__device__ __forceinline__ Cx<T> cmul(Cx<T> a, Cx<T> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T>
__device__ __forceinline__ Cx<T> cel(const M3<T>& a, int k) {
    return {a.r[k], a.i[k]};
}
template <typename T>
__device__ __forceinline__ Cx<T> csub(Cx<T> a, Cx<T> b) {
    return {a.re - b.re, a.im - b.im};
}

// Relative truncation tolerance of the series: a term whose bound
// |A|_F^k / k! is below tol |A|_F is dropped together with every later one
// (their sum is < 1.2 x the bound for |A|_F <= 1/2).
template <typename T>
__device__ __forceinline__ T exp_tol();
template <>
__device__ __forceinline__ float exp_tol<float>() {
    return 1.5e-8f;  // ~2^-26
}
template <>
__device__ __forceinline__ double exp_tol<double>() {
    return 2.8e-17;  // ~2^-55
}

// exp(A) - I of a 3x3 complex matrix.  Cayley-Hamilton, A^3 = t A^2 - m A + d I
// with t = tr A, m = (t^2 - tr A^2)/2, d = det A, gives
// A^k = p_k I + q_k A + r_k A^2 with (p, q, r)_{k+1} = (d r_k, p_k - m r_k,
// q_k + t r_k), so the Taylor series costs one matrix product (A^2) and scalar
// recurrences:
//     exp A - I = (sum_{k>=3} p_k/k!) I + (sum q_k/k!) A + (sum r_k/k!) A^2.
// p_k, q_k, r_k are divided differences of x^k over the eigenvalues, bounded by
// k^2 |A|^(k-2), so the sum is stable at |A|_F <= 1/2; larger arguments are
// scaled by 2^-s and squared back s times as D <- 2 D + D D.
template <typename T>
__device__ __forceinline__ M3<T> expm1_m3(const M3<T>& x) {
    T nrm = T(0);
#pragma unroll
    for (int k = 0; k < 9; ++k) nrm += x.r[k] * x.r[k] + x.i[k] * x.i[k];
    nrm = sqrt(nrm);
    int sq = 0;
    T sc = T(1);
    while (nrm * sc > T(0.5) && sq < 60) {
        sc *= T(0.5);
        ++sq;
    }
    const M3<T> a = m_scale(x, sc);
    nrm *= sc;
    const M3<T> a2 = mul(a, a);
    const Cx<T> t = {a.r[0] + a.r[4] + a.r[8], a.i[0] + a.i[4] + a.i[8]};
    const Cx<T> tr2 = {a2.r[0] + a2.r[4] + a2.r[8], a2.i[0] + a2.i[4] + a2.i[8]};
    Cx<T> m = cmul(t, t);
    m = {T(0.5) * (m.re - tr2.re), T(0.5) * (m.im - tr2.im)};
    const Cx<T> d0 = cmul(cel(a, 0), csub(cmul(cel(a, 4), cel(a, 8)), cmul(cel(a, 5), cel(a, 7))));
    const Cx<T> d1 = cmul(cel(a, 1), csub(cmul(cel(a, 3), cel(a, 8)), cmul(cel(a, 5), cel(a, 6))));
    const Cx<T> d2 = cmul(cel(a, 2), csub(cmul(cel(a, 3), cel(a, 7)), cmul(cel(a, 4), cel(a, 6))));
    const Cx<T> d = {d0.re - d1.re + d2.re, d0.im - d1.im + d2.im};
    // terms k = 1, 2: A + A^2/2; state (p, q, r) of A^2
    Cx<T> s0 = {T(0), T(0)}, s1 = {T(1), T(0)}, s2 = {T(0.5), T(0)};
    Cx<T> p = {T(0), T(0)}, q = {T(0), T(0)}, r = {T(1), T(0)};
    T f = T(0.5), bnd = T(0.5) * nrm * nrm;
    const T tol = exp_tol<T>() * nrm;
    for (int k = 3; k <= 40; ++k) {
        bnd *= nrm / T(k);
        if (!(bnd > tol)) break;
        const Cx<T> rd = cmul(r, d), rm = cmul(r, m), rt = cmul(r, t);
        const Cx<T> pn = rd, qn = csub(p, rm), rn = {q.re + rt.re, q.im + rt.im};
        p = pn;
        q = qn;
        r = rn;
        f /= T(k);
        s0.re += f * p.re;
        s0.im += f * p.im;
        s1.re += f * q.re;
        s1.im += f * q.im;
        s2.re += f * r.re;
        s2.im += f * r.im;
    }
    M3<T> e;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        e.r[k] = s1.re * a.r[k] - s1.im * a.i[k] + s2.re * a2.r[k] - s2.im * a2.i[k];
        e.i[k] = s1.re * a.i[k] + s1.im * a.r[k] + s2.re * a2.i[k] + s2.im * a2.r[k];
    }
#pragma unroll
    for (int k = 0; k < 9; k += 4) {
        e.r[k] += s0.re;
        e.i[k] += s0.im;
    }
    for (int k = 0; k < sq; ++k) {
        M3<T> dd = mul(e, e);
        m_axpy(dd, T(2), e);
        e = dd;
    }
    return e;
}

template <typename T>
__device__ __forceinline__ M3<T> load_full(const void* links, int64_t V, int64_t s, int mu) {
    using C2 = typename V2<T>::type;
    if (!FLUE_INB(s >= 0 && s < V && mu >= 0 && mu < 4)) return m_zero<T>();
    const C2* q = (const C2*)links + s + V * mu;
    M3<T> m;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const C2 v = q[4 * V * (a + 3 * b)];
            m.r[3 * a + b] = v.x;
            m.i[3 * a + b] = v.y;
        }
    return m;
}

// Float-float accumulator of products: hi + lo holds the sum to ~2^-48
// (error-free products by fma, Knuth's two-sum; the _rn intrinsics keep the
// compiler from contracting them).
struct FF {
    float hi, lo;
};
__device__ __forceinline__ void ff_addprod(FF& s, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = fmaf(a, b, -p);
    const float t = __fadd_rn(s.hi, p);
    const float bp = __fsub_rn(t, s.hi);
    const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s.hi = t;
    s.lo = __fadd_rn(s.lo, __fadd_rn(err, e));
}

// Row r of length^2 1 + delta -> r (1 + c), c = (1 + delta)^-1/2 - 1, with
// delta from the float-float sum so the row is rounded once.
__device__ __forceinline__ void ff_normalise(float r[3], float i[3]) {
    FF n{0.f, 0.f};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        ff_addprod(n, r[c], r[c]);
        ff_addprod(n, i[c], i[c]);
    }
    const float d = __fadd_rn(__fsub_rn(n.hi, 1.0f), n.lo);
    const float c = fabsf(d) < 1e-3f ? d * (-0.5f + d * (0.375f - 0.3125f * d)) : rsqrtf(1.0f + d) - 1.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        r[k] = fmaf(c, r[k], r[k]);
        i[k] = fmaf(c, i[k], i[k]);
    }
}

// FixSU3Matrix (row 0 normalised, row 1 orthogonalised and normalised,
// row 2 = conj(row0 x row1) normalised) in FP32.  The norms, the overlap and
// the cross products are small differences of O(1) products; summing them in
// float-float leaves one rounding per entry, as FP64 arithmetic rounded to
// FP32 would.  With plain FP32 sums the flowed B^2 of a 32^3x64 field
// drifted from the FP64 flow by 2.8e-6 (relative) after 200 steps of 0.01;
// with these sums by 9.5e-8, the same as with FixSU3Matrix in FP64.
__device__ __forceinline__ void fix_su3_rows_f32(float r[3][3], float i[3][3]) {
    ff_normalise(r[0], i[0]);
    FF dr{0.f, 0.f}, di{0.f, 0.f};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        ff_addprod(dr, r[0][c], r[1][c]);
        ff_addprod(dr, i[0][c], i[1][c]);
        ff_addprod(di, r[0][c], i[1][c]);
        ff_addprod(di, -i[0][c], r[1][c]);
    }
    const float ovr = dr.hi + dr.lo, ovi = di.hi + di.lo;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        r[1][c] -= r[0][c] * ovr - i[0][c] * ovi;
        i[1][c] -= r[0][c] * ovi + i[0][c] * ovr;
    }
    ff_normalise(r[1], i[1]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int j = (c + 1) % 3, k = (c + 2) % 3;
        FF re{0.f, 0.f}, im{0.f, 0.f};
        ff_addprod(re, r[0][j], r[1][k]);
        ff_addprod(re, -i[0][j], i[1][k]);
        ff_addprod(re, -r[0][k], r[1][j]);
        ff_addprod(re, i[0][k], i[1][j]);
        ff_addprod(im, r[0][j], i[1][k]);
        ff_addprod(im, i[0][j], r[1][k]);
        ff_addprod(im, -r[0][k], i[1][j]);
        ff_addprod(im, -i[0][k], r[1][j]);
        r[2][c] = re.hi + re.lo;
        i[2][c] = -(im.hi + im.lo);
    }
    ff_normalise(r[2], i[2]);
}

template <typename W>
__device__ __forceinline__ void reunitarise(M3<W>& w) {
    W r[3][3], im[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            r[a][b] = w.r[3 * a + b];
            im[a][b] = w.i[3 * a + b];
        }
    if constexpr (sizeof(W) == 4)
        fix_su3_rows_f32(r, im);
    else
        fix_su3_rows(r, im);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            w.r[3 * a + b] = r[a][b];
            w.i[3 * a + b] = im[a][b];
        }
}

template <typename T>
__global__ void k_wflow_update(void* links, Geom g, const void* force, AHPlanes<T> bbuf, T eps, int stage,
                               int reun) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 4 * g.V) return;
    const int64_t s = idx % g.V;
    const int mu = (int)(idx / g.V);
    // Z = eps * 2 G, G in the field's compute type, same layout as the field
    M3<T> z = load_full<T>(force, g.V, s, mu);
    z = m_scale(z, T(2) * eps);
    M3<T> x;
    if (stage == 0) {
        bbuf.store(s, mu, z);
        x = m_scale(z, T(0.25));
    } else if (stage == 1) {
        const M3<T> b = bbuf.load(s, mu);
        x = m_scale(z, T(8.0 / 9.0));
        m_axpy(x, T(-17.0 / 36.0), b);
        bbuf.store(s, mu, x);
    } else {
        const M3<T> b = bbuf.load(s, mu);
        x = m_scale(z, T(0.75));
        m_axpy(x, T(-1), b);
    }
    const M3<T> dm = expm1_m3(x);
    const M3<T> u = load_full<T>(links, g.V, s, mu);
    M3<T> w = mul(dm, u);
    m_axpy(w, T(1), u);
    if (reun) reunitarise(w);
    using C2 = typename V2<T>::type;
    C2* q = (C2*)links + s + g.V * mu;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            C2 v;
            v.x = w.r[3 * a + b];
            v.y = w.i[3 * a + b];
            q[4 * g.V * (a + 3 * b)] = v;
        }
}

cudaError_t launch_wflow_step(void* links, const Geom& g, int prec, double eps, void* ws, cudaStream_t st) {
    char* w = (char*)ws;
    const size_t f = (((size_t)36 * g.V * 16) + 255) & ~(size_t)255;
    const size_t b = (((size_t)36 * g.V * 8) + 255) & ~(size_t)255;
    void* force = w;
    // B in the field's precision (the slot is sized for FP64)
    AHPlanes<double> bb{(double*)(w + f), g.V};
    AHPlanes<float> bbf{(float*)(w + f), g.V};
    double* part = (double*)(w + f + b);
    FieldRef U{links, g, prec};
    const unsigned nb = (unsigned)((4 * g.V + 127) / 128);
    for (int stage = 0; stage < 3; ++stage) {
        cudaError_t e = launch_plaquette_force(U, part, nullptr, force, 0, st);
        if (e != cudaSuccess) return e;
        if (prec == PREC_C128)
            note_launch(), k_wflow_update<double><<<nb, 128, 0, st>>>(links, g, force, bb, eps, stage, 0);
        else
            note_launch(), k_wflow_update<float><<<nb, 128, 0, st>>>(links, g, force, bbf, (float)eps, stage, 1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

FLUE_OOB_READER(flow)

}  // namespace flue
