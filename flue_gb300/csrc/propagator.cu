// propagator.cu -- gauge transformation of a device field and the scalar
// gluon propagator D(q) on every lattice momentum.
//
// The reference's propagator routines (src/gluonCalc/gluonProp.f90) are
// unfinished: calc_mom_space_scalarD reads U(N - q) outside its declared
// (0:N) bounds at q = 0 and tests q = 0 as `qx + qy + qx < 1`;
// scalarGluonProp's Fourier sums ignore their own loop indices; colourDecomp
// (src/SU3MatrixOps.f90:107-122) keeps only real parts of the off-diagonal
// sums.  What they work towards is the standard lattice definition of
// hep-lat/9803105 (cited at gluonProp.f90:38), which is computed here:
//
//   A_mu(x) = [U_mu(x) - U_mu(x)^+]/(2i) - trace/3      (traceless Hermitian)
//   A^a_mu(x) = Tr(A_mu(x) lambda^a)                       (8 real fields)
//   A^a_mu(q) = sum_x exp(-i q.x) A^a_mu(x),  q_mu = 2 pi n_mu / N_mu
//   D(q) = sum_{mu >= mu_start} w_mu sum_a |A^a_mu(q)|^2 / ((Nc^2-1) n(q) V)
//
// with w_t = xi^2, w_i = 1 (gluonProp.f90:186-190), n(0) = 4, n(q != 0) = 3
// (the longitudinal part vanishes in Landau gauge; gluonProp.f90:208-236).
// Since A = sum_a A^a lambda^a / 2, sum_a |A^a(q)|^2 = 2 Tr(A(q) A(-q)) and
// D(q) = 2/((Nc^2-1) n V) sum_mu Tr<A_mu(q) A_mu(-q)>, the paper's form.
// The midpoint phase exp(-i q_mu / 2) has modulus 1 and drops out of D.
//
// Pipeline: k_colour_fields writes the 32 real fields A^a_mu(x) (t fastest;
// component-major [mu,a][x,y,z][t] for FP32, site-major [x,y,z][mu,a][t] for
// FP64, see prop_cmajor); cuFFT transforms t (real to complex, NT/2+1
// outputs) and then (x,y,z) in one batched complex transform over all 32
// components and time frequencies; k_prop_sum adds |A^a_mu(q)|^2 per
// momentum, taking q_t > NT/2 from -q by the real fields' Hermitian
// symmetry.  cuFFT runs in the field's compute precision (FP64 for c128,
// FP32 for c64/r12); the sums are FP64.
#include <cufft.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <tuple>

#include "flue_internal.h"

namespace flue {

// ---------------------------------------------------------------------------
// gauge transformation in place: U_mu(x) <- G(x) U_mu(x) G(x+mu)^+
// ---------------------------------------------------------------------------
template <typename T, typename G2>
__device__ __forceinline__ M3<T> load_gt(const G2* __restrict__ G, int64_t V, int64_t s) {
    M3<T> m;
    if (!FLUE_INB(s >= 0 && s < V)) return m_zero<T>();
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const G2 v = G[s + V * (a + 3 * b)];
            m.r[3 * a + b] = (T)v.x;
            m.i[3 * a + b] = (T)v.y;
        }
    return m;
}

template <class L, typename T, typename G2>
__global__ void k_gauge_transform(L U, void* links, int prec, Geom g, const G2* __restrict__ G) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 4 * g.V) return;
    const int64_t s = idx % g.V;
    const int mu = (int)(idx / g.V);
    int c[4];
    site_coords(g, s, c);
    int64_t sp = s;  // x + mu, selected without runtime-indexed arrays
#pragma unroll
    for (int d = 0; d < 4; ++d)
        if (d == mu) sp = s + (c[d] + 1 == g.n[d] ? -(int64_t)(g.n[d] - 1) * g.st[d] : g.st[d]);
    const M3<T> gx = load_gt<T>(G, g.V, s);
    const M3<T> gp = load_gt<T>(G, g.V, sp);
    const M3<T> w = mm<false, true>(mul(gx, U.load(s, mu)), gp);
    if (prec == PREC_R12) {
        float4* o = (float4*)links + s + g.V * (3 * mu);
        o[0] = make_float4(w.r[0], w.i[0], w.r[1], w.i[1]);
        o[g.V] = make_float4(w.r[2], w.i[2], w.r[3], w.i[3]);
        o[2 * g.V] = make_float4(w.r[4], w.i[4], w.r[5], w.i[5]);
    } else {
        using C2 = typename V2<T>::type;
        C2* o = (C2*)links + s + g.V * mu;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                C2 v;
                v.x = w.r[3 * a + b];
                v.y = w.i[3 * a + b];
                o[4 * g.V * (a + 3 * b)] = v;
            }
    }
}

cudaError_t launch_gauge_transform(const FieldRef& U, const void* G, int g_dtype, cudaStream_t st) {
    const unsigned nb = (unsigned)((4 * U.g.V + 127) / 128);
    void* links = const_cast<void*>(U.links);
    FLUE_DISPATCH_LINKS(U, {
        if (g_dtype == PREC_C128)
            note_launch(), k_gauge_transform<decltype(L), T, double2>
                               <<<nb, 128, 0, st>>>(L, links, U.prec, U.g, (const double2*)G);
        else
            note_launch(), k_gauge_transform<decltype(L), T, float2>
                               <<<nb, 128, 0, st>>>(L, links, U.prec, U.g, (const float2*)G);
    });
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 1. colour components A^a_mu(x), written as a[((s3 * 32) + 8 mu + a) * NT + t]
// ---------------------------------------------------------------------------
// With A = (U - U^+)/(2i): A_ij = (U_ij - conj U_ji)/(2i), so
// 2 Re A_ij = Im U_ij + Im U_ji, 2 Im A_ij = Re U_ji - Re U_ij, A_ii = Im U_ii.
// The trace part drops out of every projection Tr(A lambda^a).
template <class L, typename T>
__global__ void k_colour_fields(L U, Geom g, int cmajor, T* __restrict__ a) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 4 * g.V) return;
    const int64_t s = idx % g.V;
    const int mu = (int)(idx / g.V);
    const M3<T> u = U.load(s, mu);
    const int64_t nt = g.n[0];
    const int64_t t = s % nt, s3 = s / nt;
    if (!FLUE_INB(s >= 0 && s < g.V && mu >= 0 && mu < 4)) return;  // 32 V outputs
    // component-major a[(c * V3 + s3) * NT + t], or site-major a[(s3 * 32 + c) * NT + t]
    const int64_t cs = cmajor ? g.V : nt;
    T* o = cmajor ? a + (8 * mu) * cs + s3 * nt + t : a + (s3 * 32 + 8 * mu) * nt + t;
    const T r3 = (T)0.57735026918962576451;  // 1/sqrt(3)
    o[0] = u.i[1] + u.i[3];                      // lambda_1: 2 Re A_12
    o[cs] = u.r[1] - u.r[3];                     // lambda_2: -2 Im A_12
    o[2 * cs] = u.i[0] - u.i[4];                 // lambda_3: A_11 - A_22
    o[3 * cs] = u.i[2] + u.i[6];                 // lambda_4: 2 Re A_13
    o[4 * cs] = u.r[2] - u.r[6];                 // lambda_5: -2 Im A_13
    o[5 * cs] = u.i[5] + u.i[7];                 // lambda_6: 2 Re A_23
    o[6 * cs] = u.r[5] - u.r[7];                 // lambda_7: -2 Im A_23
    o[7 * cs] = (u.i[0] + u.i[4] - T(2) * u.i[8]) * r3;  // lambda_8
}

// ---------------------------------------------------------------------------
// 3. D(q) from the transformed fields F[((s3 * 32) + c) * nth + kt], one
//    thread per element of the half spectrum kt <= NT/2: it reads the 32
//    components once and writes D(q) and, for 0 < kt < NT - kt, D(-q)
//    (|A(-q)| = |A(q)| for real fields)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_prop_sum(const typename V2<T>::type* __restrict__ F, Geom g, int nth, int cmajor, double xi2,
                           int mu_start, double* __restrict__ D) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t v3 = g.V / g.n[0];
    if (idx >= v3 * nth) return;
    // spectrum F[(c * nth + kt) * V3 + s3] (component-major) or
    // F[(s3 * 32 + c) * nth + kt]; consecutive threads read consecutive entries
    const int64_t s3 = cmajor ? idx % v3 : idx / nth;
    const int kt = (int)(cmajor ? idx / v3 : idx % nth);
    const typename V2<T>::type* f = cmajor ? F + kt * v3 + s3 : F + s3 * 32 * nth + kt;
    const int64_t fs = cmajor ? (int64_t)nth * v3 : nth;  // component stride
    double sum = 0.0;
    if (!FLUE_INB(s3 >= 0 && s3 < v3 && kt >= 0 && kt < nth)) return;  // F holds 32 * v3 * nth
    for (int mu = mu_start; mu < 4; ++mu) {
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const typename V2<T>::type c = f[(int64_t)(8 * mu + a) * fs];
            s += (double)c.x * (double)c.x + (double)c.y * (double)c.y;
        }
        sum += (mu == 0 ? xi2 : 1.0) * s;
    }
    const double norm = 1.0 / (8.0 * 3.0 * (double)g.V);
    const int nt = g.n[0];
    const bool q0 = kt == 0 && s3 == 0;
    D[kt + (int64_t)nt * s3] = q0 ? sum / (8.0 * 4.0 * (double)g.V) : sum * norm;
    if (kt > 0 && kt < nt - kt) {
        const int kx = (int)(s3 % g.n[1]), ky = (int)((s3 / g.n[1]) % g.n[2]), kz = (int)(s3 / ((int64_t)g.n[1] * g.n[2]));
        const int mx = kx ? g.n[1] - kx : 0, my = ky ? g.n[2] - ky : 0, mz = kz ? g.n[3] - kz : 0;
        const int64_t m3 = mx + (int64_t)g.n[1] * (my + (int64_t)g.n[2] * mz);
        D[(nt - kt) + (int64_t)nt * m3] = sum * norm;
    }
}

// ---------------------------------------------------------------------------
// cuFFT plans, cached per (device, extents, precision); the work area comes
// from the caller's workspace (auto-allocation off)
// ---------------------------------------------------------------------------
// Layout of the colour fields and spectrum: component-major for FP32
// transforms (the (z,y,x) transforms are then contiguous batched 3-D FFTs:
// 32^3x64 1.69 -> 1.16 ms per propagator), site-major for FP64 (its strided
// transforms measured faster: 5.88 against 6.29 ms).
__host__ __device__ inline bool prop_cmajor(bool dbl) { return !dbl; }

namespace {
struct PropPlans {
    cufftHandle t = 0, xyz = 0;
    size_t work = 0;
};
std::mutex g_plan_mtx;
std::map<std::tuple<int, int, int, int, int, int>, PropPlans> g_plans;

cudaError_t cufft_error(cufftResult r) {
    if (r == CUFFT_SUCCESS) return cudaSuccess;
    char msg[96];
    snprintf(msg, sizeof(msg), "cuFFT error %d", (int)r);
    set_error_detail(msg);
    return r == CUFFT_ALLOC_FAILED ? cudaErrorMemoryAllocation : cudaErrorUnknown;
}

// plans for geometry g; caller holds g_plan_mtx
cudaError_t get_plans(const Geom& g, bool dbl, PropPlans** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_tuple(dev, g.n[0], g.n[1], g.n[2], g.n[3], (int)dbl);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
        *out = &it->second;
        return cudaSuccess;
    }
    PropPlans p;
    const long long nt = g.n[0], nth = nt / 2 + 1, v3 = g.V / nt;
    const bool cmajor = prop_cmajor(dbl);
    size_t w1 = 0, w2 = 0;
    cufftResult r = cufftCreate(&p.t);
    if (r == CUFFT_SUCCESS) r = cufftCreate(&p.xyz);
    if (r == CUFFT_SUCCESS) r = cufftSetAutoAllocation(p.t, 0);
    if (r == CUFFT_SUCCESS) r = cufftSetAutoAllocation(p.xyz, 0);
    // time: real to complex along the contiguous t, one transform per
    // (spatial site, component)
    long long n1[1] = {nt}, in1[1] = {nt}, on1[1] = {nth};
    if (r == CUFFT_SUCCESS) {
        if (cmajor)  // one component per execution: element kt of row s3 at kt * V3 + s3
            r = cufftMakePlanMany64(p.t, 1, n1, in1, 1, nt, on1, v3, 1, dbl ? CUFFT_D2Z : CUFFT_R2C, v3, &w1);
        else
            r = cufftMakePlanMany64(p.t, 1, n1, in1, 1, nt, on1, 1, nth, dbl ? CUFFT_D2Z : CUFFT_R2C, v3 * 32, &w1);
    }
    // space: complex (z, y, x) transform, element stride 32 * nth, one
    // transform per (component, time frequency): batch index = offset
    long long n3[3] = {g.n[3], g.n[2], g.n[1]};
    if (r == CUFFT_SUCCESS) {
        if (cmajor)  // contiguous (z, y, x) transforms, one per (component, time frequency)
            r = cufftMakePlanMany64(p.xyz, 3, n3, n3, 1, v3, n3, 1, v3, dbl ? CUFFT_Z2Z : CUFFT_C2C, 32 * nth, &w2);
        else  // element stride 32 nth, one transform per (component, time frequency) at offset b
            r = cufftMakePlanMany64(p.xyz, 3, n3, n3, 32 * nth, 1, n3, 32 * nth, 1, dbl ? CUFFT_Z2Z : CUFFT_C2C,
                                    32 * nth, &w2);
    }
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(p.t);
        cufftDestroy(p.xyz);
        return cufft_error(r);
    }
    p.work = w1 > w2 ? w1 : w2;
    auto res = g_plans.emplace(key, p);
    *out = &res.first->second;
    return cudaSuccess;
}

inline size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

struct PropWs {
    size_t comp, spec, work, total;
};
PropWs prop_layout(const Geom& g, bool dbl, size_t work) {
    const size_t es = dbl ? 8 : 4;
    const size_t nth = g.n[0] / 2 + 1, v3 = g.V / g.n[0];
    PropWs w;
    w.comp = 0;
    w.spec = a256((size_t)32 * g.V * es);
    w.work = w.spec + a256((size_t)32 * v3 * nth * 2 * es);
    w.total = w.work + a256(work);
    return w;
}
}  // namespace

// Scratch of the propagator: the 32 real fields, their spectrum and the
// cuFFT work area (queried from the plans on the current device; without a
// usable device, the spectrum size stands in for the work area).
size_t gluon_prop_ws_bytes(const Geom& g, int prec) {
    const bool dbl = prec == PREC_C128;
    size_t work = 0;
    {
        std::lock_guard<std::mutex> lk(g_plan_mtx);
        PropPlans* p = nullptr;
        if (get_plans(g, dbl, &p) == cudaSuccess) {
            work = p->work;
        } else {
            cudaGetLastError();
            const size_t nth = g.n[0] / 2 + 1;
            work = (size_t)32 * (g.V / g.n[0]) * nth * 2 * (dbl ? 8 : 4);
        }
    }
    return prop_layout(g, dbl, work).total;
}

cudaError_t launch_gluon_propagator(const FieldRef& U, double xi, int mu_start, double* D, void* ws, size_t ws_bytes,
                                    cudaStream_t st) {
    const bool dbl = U.prec == PREC_C128;
    const Geom& g = U.g;
    std::lock_guard<std::mutex> lk(g_plan_mtx);
    PropPlans* p = nullptr;
    cudaError_t e = get_plans(g, dbl, &p);
    if (e != cudaSuccess) return e;
    const PropWs w = prop_layout(g, dbl, p->work);
    if (ws_bytes < w.total) return cudaErrorInvalidValue;
    char* base = (char*)ws;
    const unsigned nb = (unsigned)((4 * g.V + 127) / 128);
    FLUE_DISPATCH_LINKS(U, {
        note_launch(), k_colour_fields<decltype(L), T><<<nb, 128, 0, st>>>(L, g, (int)prop_cmajor(dbl), (T*)(base + w.comp));
    });
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // the plans are shared: stream and work area are set and the transforms
    // enqueued under the plan lock
    cufftResult r = cufftSetStream(p->t, st);
    if (r == CUFFT_SUCCESS) r = cufftSetStream(p->xyz, st);
    if (r == CUFFT_SUCCESS) r = cufftSetWorkArea(p->t, base + w.work);
    if (r == CUFFT_SUCCESS) r = cufftSetWorkArea(p->xyz, base + w.work);
    const bool cm = prop_cmajor(dbl);
    const int64_t v3 = cm ? g.V / g.n[0] : 0, nthl = cm ? g.n[0] / 2 + 1 : 0;
    const int ncomp_exec = cm ? 32 : 1;  // component-major: one time transform per component
    if (dbl) {
        for (int c = 0; c < ncomp_exec && r == CUFFT_SUCCESS; ++c)
            r = cufftExecD2Z(p->t, (cufftDoubleReal*)(base + w.comp) + c * v3 * g.n[0],
                             (cufftDoubleComplex*)(base + w.spec) + c * nthl * v3);
        if (r == CUFFT_SUCCESS)
            r = cufftExecZ2Z(p->xyz, (cufftDoubleComplex*)(base + w.spec), (cufftDoubleComplex*)(base + w.spec),
                             CUFFT_FORWARD);
    } else {
        for (int c = 0; c < ncomp_exec && r == CUFFT_SUCCESS; ++c)
            r = cufftExecR2C(p->t, (cufftReal*)(base + w.comp) + c * v3 * g.n[0],
                             (cufftComplex*)(base + w.spec) + c * nthl * v3);
        if (r == CUFFT_SUCCESS)
            r = cufftExecC2C(p->xyz, (cufftComplex*)(base + w.spec), (cufftComplex*)(base + w.spec), CUFFT_FORWARD);
    }
    if (r != CUFFT_SUCCESS) return cufft_error(r);
    note_launch(2);  // the two transforms (cuFFT may split each into several kernels)
    const int nth = g.n[0] / 2 + 1;
    const unsigned nq = (unsigned)(((g.V / g.n[0]) * nth + 127) / 128);
    if (dbl)
        note_launch(), k_prop_sum<double>
                           <<<nq, 128, 0, st>>>((const double2*)(base + w.spec), g, nth, (int)prop_cmajor(true), xi * xi, mu_start, D);
    else
        note_launch(), k_prop_sum<float>
                           <<<nq, 128, 0, st>>>((const float2*)(base + w.spec), g, nth, (int)prop_cmajor(false), xi * xi, mu_start, D);
    return cudaGetLastError();
}

FLUE_OOB_READER(propagator)

}  // namespace flue
