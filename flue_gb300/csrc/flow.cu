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
// exp of the traceless anti-Hermitian X is evaluated in FP64 by scaling and
// squaring with a degree-12 Taylor polynomial (Moler & Van Loan, "Nineteen
// dubious ways to compute the exponential of a matrix", method 3).  FP32
// fields are reunitarised (FixSU3Matrix) after every stage.
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

__device__ __forceinline__ M3<double> exp_su3(const M3<double>& x) {
    double nrm = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) nrm += x.r[k] * x.r[k] + x.i[k] * x.i[k];
    nrm = sqrt(nrm);
    int sq = 0;
    double sc = 1.0;
    while (nrm * sc > 0.25 && sq < 40) {
        sc *= 0.5;
        ++sq;
    }
    const M3<double> a = m_scale(x, sc);
    // Horner: I + a(I + a/2(I + a/3(... (I + a/12))))
    M3<double> p = m_ident<double>();
    for (int k = 12; k >= 1; --k) {
        M3<double> t = mul(a, p);
        t = m_scale(t, 1.0 / (double)k);
        t.r[0] += 1.0;
        t.r[4] += 1.0;
        t.r[8] += 1.0;
        p = t;
    }
    for (int k = 0; k < sq; ++k) p = mul(p, p);
    return p;
}

template <typename T>
__device__ __forceinline__ M3<double> load_full(const void* links, int64_t V, int64_t s, int mu) {
    using C2 = typename V2<T>::type;
    const C2* q = (const C2*)links + s + V * mu;
    M3<double> m;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const C2 v = q[4 * V * (a + 3 * b)];
            m.r[3 * a + b] = (double)v.x;
            m.i[3 * a + b] = (double)v.y;
        }
    return m;
}

template <typename T>
__global__ void k_wflow_update(void* links, Geom g, const void* force, AHPlanes<double> bbuf, double eps, int stage,
                               int reun) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 4 * g.V) return;
    const int64_t s = idx % g.V;
    const int mu = (int)(idx / g.V);
    // Z = eps * 2 G, G in the field's compute type, same layout as the field
    M3<double> z = load_full<T>(force, g.V, s, mu);
    z = m_scale(z, 2.0 * eps);
    M3<double> x;
    if (stage == 0) {
        bbuf.store(s, mu, z);
        x = m_scale(z, 0.25);
    } else if (stage == 1) {
        const M3<double> b = bbuf.load(s, mu);
        x = m_scale(z, 8.0 / 9.0);
        m_axpy(x, -17.0 / 36.0, b);
        bbuf.store(s, mu, x);
    } else {
        const M3<double> b = bbuf.load(s, mu);
        x = m_scale(z, 0.75);
        m_axpy(x, -1.0, b);
    }
    const M3<double> e = exp_su3(x);
    const M3<double> u = load_full<T>(links, g.V, s, mu);
    M3<double> w = mul(e, u);
    if (reun) {
        double r[3][3], im[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                r[a][b] = w.r[3 * a + b];
                im[a][b] = w.i[3 * a + b];
            }
        fix_su3_rows(r, im);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                w.r[3 * a + b] = r[a][b];
                w.i[3 * a + b] = im[a][b];
            }
    }
    using C2 = typename V2<T>::type;
    C2* q = (C2*)links + s + g.V * mu;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            C2 v;
            v.x = (T)w.r[3 * a + b];
            v.y = (T)w.i[3 * a + b];
            q[4 * g.V * (a + 3 * b)] = v;
        }
}

cudaError_t launch_wflow_step(void* links, const Geom& g, int prec, double eps, void* ws, cudaStream_t st) {
    char* w = (char*)ws;
    const size_t f = (((size_t)36 * g.V * 16) + 255) & ~(size_t)255;
    const size_t b = (((size_t)36 * g.V * 8) + 255) & ~(size_t)255;
    void* force = w;
    AHPlanes<double> bb{(double*)(w + f), g.V};
    double* part = (double*)(w + f + b);
    FieldRef U{links, g, prec};
    const unsigned nb = (unsigned)((4 * g.V + 127) / 128);
    for (int stage = 0; stage < 3; ++stage) {
        cudaError_t e = launch_plaquette_force(U, part, nullptr, force, 0, st);
        if (e != cudaSuccess) return e;
        if (prec == PREC_C128)
            k_wflow_update<double><<<nb, 128, 0, st>>>(links, g, force, bb, eps, stage, 0);
        else
            k_wflow_update<float><<<nb, 128, 0, st>>>(links, g, force, bb, eps, stage, 1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace flue
