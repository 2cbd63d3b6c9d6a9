// flue_common.cuh -- device-side building blocks shared by every kernel.
//
//  * M3<T>: a 3x3 complex matrix held in registers as 9 real + 9 imaginary
//    parts (row-major, element (a,b) at 3a+b).  T = double for the FP64
//    path, float for the FP32 path.  The products are the 3x3 complex algebra
//    of src/SU3MatrixOps.f90 (MultiplyMatMat :19-37, MultiplyMatdagMatdag
//    :39-58, traces :60-92) written as FMA chains, with the dagger of either
//    operand folded into the index pattern at compile time.
//  * Link storage on the device ("field layouts"):
//      - FULL (complex128 or complex64): exactly the reference's Fortran
//        array data(NT,NX,NY,NZ,4,3,3) (src/wloops.F90:60): complex element
//        (s, mu, a, b) at offset s + V*(mu + 4*(a + 3*b)).  Every colour
//        component is a site-fastest plane, so a warp reading 32 consecutive
//        sites issues fully coalesced 16-byte (c128) or 8-byte (c64) loads.
//      - R12 (float): the first two rows only, as three float4 planes per
//        direction: float4 (mu, k) of site s at s + V*(k + 3*mu), k = 0:
//        (U00,U01), 1: (U02,U10), 2: (U11,U12).  The third row is rebuilt as
//        conj(row0 x row1), the vector_product of FixSU3Matrix
//        (src/gaugeIO/ILDG_bin.f90:120-135, :146).  48 bytes per link with
//        128-bit coalesced loads.
//  * Geometry: sites are numbered t-fastest, s = t + NT*(x + NX*(y + NY*z)),
//    direction index mu = 0,1,2,3 <-> t,x,y,z (the reference's 1..4).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Bounds-checked build (-DFLUE_BOUNDS_CHECK=1): the link and intermediate
// accessors check every index, count violations in a device counter of the
// translation unit and skip the access (loads return zeros) -- no trap, no
// fault.  flue_bounds_errors() reads and clears the counters.  Off by default.
#ifndef FLUE_BOUNDS_CHECK
#define FLUE_BOUNDS_CHECK 0
#endif

namespace flue {

#if FLUE_BOUNDS_CHECK
namespace {
__device__ unsigned int g_oob_count;  // one per translation unit
}
__device__ __forceinline__ bool in_bounds(bool ok) {
    if (!ok) atomicAdd(&g_oob_count, 1u);
    return ok;
}
// read and clear this translation unit's counter (host)
static inline unsigned oob_read_clear() {
    unsigned v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, g_oob_count, sizeof(v)) != cudaSuccess) return 0xffffffffu;
    cudaMemcpyToSymbol(g_oob_count, &z, sizeof(z));
    return v;
}
#define FLUE_INB(cond) ::flue::in_bounds(cond)
#else
static inline unsigned oob_read_clear() { return 0; }
#define FLUE_INB(cond) true
#endif
// per translation unit: unsigned flue::oob_<name>() for flue_bounds_errors()
#define FLUE_OOB_READER(name) \
    unsigned oob_##name() { return oob_read_clear(); }

enum Prec : int { PREC_C128 = 0, PREC_C64 = 1, PREC_R12 = 2 };

template <typename T>
struct V2;
template <>
struct V2<double> {
    using type = double2;
};
template <>
struct V2<float> {
    using type = float2;
};

template <typename T>
struct M3 {
    T r[9], i[9];
};

template <typename T>
__device__ __forceinline__ M3<T> m_zero() {
    M3<T> m;
#pragma unroll
    for (int k = 0; k < 9; ++k) m.r[k] = m.i[k] = T(0);
    return m;
}
template <typename T>
__device__ __forceinline__ M3<T> m_ident() {
    M3<T> m = m_zero<T>();
    m.r[0] = m.r[4] = m.r[8] = T(1);
    return m;
}
template <typename T>
__device__ __forceinline__ M3<T> dag(const M3<T>& a) {
    M3<T> m;
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = 0; y < 3; ++y) {
            m.r[3 * x + y] = a.r[3 * y + x];
            m.i[3 * x + y] = -a.i[3 * y + x];
        }
    return m;
}
template <typename T>
__device__ __forceinline__ M3<T> transp(const M3<T>& a) {
    M3<T> m;
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = 0; y < 3; ++y) {
            m.r[3 * x + y] = a.r[3 * y + x];
            m.i[3 * x + y] = a.i[3 * y + x];
        }
    return m;
}

// C += op(A) * op(B), op = dagger when DA / DB.
template <bool DA, bool DB, typename T>
__device__ __forceinline__ void mac(M3<T>& C, const M3<T>& A, const M3<T>& B) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            T re = C.r[3 * a + b], im = C.i[3 * a + b];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T ar = DA ? A.r[3 * k + a] : A.r[3 * a + k];
                const T ai = DA ? -A.i[3 * k + a] : A.i[3 * a + k];
                const T br = DB ? B.r[3 * b + k] : B.r[3 * k + b];
                const T bi = DB ? -B.i[3 * b + k] : B.i[3 * k + b];
                re = fma(ar, br, re);
                re = fma(-ai, bi, re);
                im = fma(ar, bi, im);
                im = fma(ai, br, im);
            }
            C.r[3 * a + b] = re;
            C.i[3 * a + b] = im;
        }
}

// C = op(A) * op(B)
template <bool DA, bool DB, typename T>
__device__ __forceinline__ M3<T> mm(const M3<T>& A, const M3<T>& B) {
    M3<T> C;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const T ar0 = DA ? A.r[a] : A.r[3 * a];
            const T ai0 = DA ? -A.i[a] : A.i[3 * a];
            const T br0 = DB ? B.r[3 * b] : B.r[b];
            const T bi0 = DB ? -B.i[3 * b] : B.i[b];
            T re = ar0 * br0;
            T im = ar0 * bi0;
            re = fma(-ai0, bi0, re);
            im = fma(ai0, br0, im);
#pragma unroll
            for (int k = 1; k < 3; ++k) {
                const T ar = DA ? A.r[3 * k + a] : A.r[3 * a + k];
                const T ai = DA ? -A.i[3 * k + a] : A.i[3 * a + k];
                const T br = DB ? B.r[3 * b + k] : B.r[3 * k + b];
                const T bi = DB ? -B.i[3 * b + k] : B.i[3 * k + b];
                re = fma(ar, br, re);
                re = fma(-ai, bi, re);
                im = fma(ar, bi, im);
                im = fma(ai, br, im);
            }
            C.r[3 * a + b] = re;
            C.i[3 * a + b] = im;
        }
    return C;
}

template <typename T>
__device__ __forceinline__ M3<T> mul(const M3<T>& A, const M3<T>& B) {
    return mm<false, false>(A, B);
}

// Re Tr(op(A) op(B))
template <bool DA, bool DB, typename T>
__device__ __forceinline__ T retr_mm(const M3<T>& A, const M3<T>& B) {
    T s = T(0);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const T ar = DA ? A.r[3 * k + a] : A.r[3 * a + k];
            const T ai = DA ? -A.i[3 * k + a] : A.i[3 * a + k];
            const T br = DB ? B.r[3 * a + k] : B.r[3 * k + a];
            const T bi = DB ? -B.i[3 * a + k] : B.i[3 * k + a];
            s = fma(ar, br, s);
            s = fma(-ai, bi, s);
        }
    return s;
}

template <typename T>
__device__ __forceinline__ T retr(const M3<T>& A) {
    return A.r[0] + A.r[4] + A.r[8];
}

template <typename T>
__device__ __forceinline__ void m_add(M3<T>& acc, const M3<T>& b) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        acc.r[k] += b.r[k];
        acc.i[k] += b.i[k];
    }
}
template <typename T>
__device__ __forceinline__ void m_axpy(M3<T>& acc, T s, const M3<T>& b) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        acc.r[k] = fma(s, b.r[k], acc.r[k]);
        acc.i[k] = fma(s, b.i[k], acc.i[k]);
    }
}
// acc += s * b^dagger
template <typename T>
__device__ __forceinline__ void m_axpy_dag(M3<T>& acc, T s, const M3<T>& b) {
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = 0; y < 3; ++y) {
            acc.r[3 * x + y] = fma(s, b.r[3 * y + x], acc.r[3 * x + y]);
            acc.i[3 * x + y] = fma(-s, b.i[3 * y + x], acc.i[3 * x + y]);
        }
}
template <typename T>
__device__ __forceinline__ M3<T> m_scale(const M3<T>& a, T s) {
    M3<T> m;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        m.r[k] = a.r[k] * s;
        m.i[k] = a.i[k] * s;
    }
    return m;
}

// Projection of cloverLoopMuNuCoord / Loop5MuNuCoord (src/wloops.F90:178-190,
// :411-423): anti-Hermitian, not traceless, times 1/4.
template <typename T>
__device__ __forceinline__ M3<T> ah_quarter(const M3<T>& u) {
    M3<T> f;
    const T h = T(0.125);  // 0.5 (projection) * 0.25 (factor)
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        f.r[4 * x] = T(0);
        f.i[4 * x] = u.i[4 * x] * T(0.25);
    }
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = x + 1; y < 3; ++y) {
            const T cr = (u.r[3 * x + y] - u.r[3 * y + x]) * h;
            const T ci = (u.i[3 * x + y] + u.i[3 * y + x]) * h;
            f.r[3 * x + y] = cr;
            f.i[3 * x + y] = ci;
            f.r[3 * y + x] = -cr;
            f.i[3 * y + x] = ci;
        }
    return f;
}

// Traceless anti-Hermitian part times s: s * [(M - M^+)/2 - Tr((M - M^+)/2)/3].
template <typename T>
__device__ __forceinline__ M3<T> ta_scaled(const M3<T>& m, T s) {
    M3<T> g;
    const T hs = T(0.5) * s;
    const T tr = (m.i[0] + m.i[4] + m.i[8]) * (T(1) / T(3));
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        g.r[4 * x] = T(0);
        g.i[4 * x] = (m.i[4 * x] - tr) * s;
    }
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = x + 1; y < 3; ++y) {
            const T cr = (m.r[3 * x + y] - m.r[3 * y + x]) * hs;
            const T ci = (m.i[3 * x + y] + m.i[3 * y + x]) * hs;
            g.r[3 * x + y] = cr;
            g.i[3 * x + y] = ci;
            g.r[3 * y + x] = -cr;
            g.i[3 * y + x] = ci;
        }
    return g;
}

// ---------------------------------------------------------------------------
// FixSU3Matrix (src/gaugeIO/ILDG_bin.f90:138-151) on rows 0 and 1; row 2
// becomes conj(row0 x row1) normalised.  Every caller that restates the
// reference runs it in FP64; the FP32 Wilson-flow update runs it in float.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void fix_su3_rows(T r[3][3], T i[3][3]) {
    // normalise row 0 (:154-159)
    T n = sqrt((r[0][0] * r[0][0] + i[0][0] * i[0][0]) + (r[0][1] * r[0][1] + i[0][1] * i[0][1]) +
                    (r[0][2] * r[0][2] + i[0][2] * i[0][2]));
    for (int c = 0; c < 3; ++c) {
        r[0][c] /= n;
        i[0][c] /= n;
    }
    // orthogonalise row 1 against row 0 (:108-118): w -= v * sum(conj(v) w)
    T dr = T(0), di = T(0);
    for (int c = 0; c < 3; ++c) {
        dr += r[0][c] * r[1][c] + i[0][c] * i[1][c];
        di += r[0][c] * i[1][c] - i[0][c] * r[1][c];
    }
    for (int c = 0; c < 3; ++c) {
        const T pr = r[0][c] * dr - i[0][c] * di, pi = r[0][c] * di + i[0][c] * dr;
        r[1][c] -= pr;
        i[1][c] -= pi;
    }
    n = sqrt((r[1][0] * r[1][0] + i[1][0] * i[1][0]) + (r[1][1] * r[1][1] + i[1][1] * i[1][1]) +
             (r[1][2] * r[1][2] + i[1][2] * i[1][2]));
    for (int c = 0; c < 3; ++c) {
        r[1][c] /= n;
        i[1][c] /= n;
    }
    // row 2 = conj(row0 x row1) (:120-135), normalised
    for (int c = 0; c < 3; ++c) {
        const int j = (c + 1) % 3, k = (c + 2) % 3;
        const T re = (r[0][j] * r[1][k] - i[0][j] * i[1][k]) - (r[0][k] * r[1][j] - i[0][k] * i[1][j]);
        const T im = (r[0][j] * i[1][k] + i[0][j] * r[1][k]) - (r[0][k] * i[1][j] + i[0][k] * r[1][j]);
        r[2][c] = re;
        i[2][c] = -im;
    }
    n = sqrt((r[2][0] * r[2][0] + i[2][0] * i[2][0]) + (r[2][1] * r[2][1] + i[2][1] * i[2][1]) +
             (r[2][2] * r[2][2] + i[2][2] * i[2][2]));
    for (int c = 0; c < 3; ++c) {
        r[2][c] /= n;
        i[2][c] /= n;
    }
}

// ---------------------------------------------------------------------------
// Link storage
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 ldg2(const double2* p) { return __ldg(p); }
__device__ __forceinline__ float2 ldg2(const float2* p) { return __ldg(p); }

// Reference layout (complex128 / complex64), read-only.
template <typename T>
struct FullLinks {
    using C2 = typename V2<T>::type;
    const C2* __restrict__ p;
    int64_t V;
    __device__ __forceinline__ M3<T> load(int64_t s, int mu) const {
        M3<T> m;
        if (!FLUE_INB(s >= 0 && s < V && mu >= 0 && mu < 4)) return m_zero<T>();
        const C2* q = p + s + V * mu;
        const int64_t st = 4 * V;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const C2 v = ldg2(q + st * (a + 3 * b));
                m.r[3 * a + b] = v.x;
                m.i[3 * a + b] = v.y;
            }
        return m;
    }
};

__device__ __forceinline__ void reconstruct_row2(M3<float>& m) {
    // row2 = conj(row0 x row1)  (vector_product of FixSU3Matrix)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int j = (c + 1) % 3, k = (c + 2) % 3;
        // v(j) w(k) - v(k) w(j) with v = row0, w = row1
        const float re = (m.r[j] * m.r[3 + k] - m.i[j] * m.i[3 + k]) - (m.r[k] * m.r[3 + j] - m.i[k] * m.i[3 + j]);
        const float im = (m.r[j] * m.i[3 + k] + m.i[j] * m.r[3 + k]) - (m.r[k] * m.i[3 + j] + m.i[k] * m.r[3 + j]);
        m.r[6 + c] = re;
        m.i[6 + c] = -im;
    }
}

struct R12Links {
    const float4* __restrict__ p;
    int64_t V;
    __device__ __forceinline__ M3<float> load(int64_t s, int mu) const {
        M3<float> m;
        if (!FLUE_INB(s >= 0 && s < V && mu >= 0 && mu < 4)) return m_zero<float>();
        const float4* q = p + s + V * (3 * mu);
        const float4 a = __ldg(q), b = __ldg(q + V), c = __ldg(q + 2 * V);
        m.r[0] = a.x;
        m.i[0] = a.y;
        m.r[1] = a.z;
        m.i[1] = a.w;
        m.r[2] = b.x;
        m.i[2] = b.y;
        m.r[3] = b.z;
        m.i[3] = b.w;
        m.r[4] = c.x;
        m.i[4] = c.y;
        m.r[5] = c.z;
        m.i[5] = c.w;
        reconstruct_row2(m);
        return m;
    }
};

// Pipeline intermediates, one matrix per (plane k, site s).
// FP32: 18 reals as 4 float4 units and 1 float2 unit (72 bytes, no padding),
// stored in tiles of 32 sites (a warp's width) with the units unit-major
// inside a tile: a tile holds 4 x 32 float4 then 32 float2 (2304 bytes, 144
// float4), tile (k, s / 32) at float4 index (k * T + s / 32) * 144, T = the
// number of tiles; float4 unit u < 4 of site s at +32 u + s % 32, the float2
// unit at float2 index 2 * (tile + 128) + s % 32.  A warp reading one unit of
// 32 consecutive sites reads 512 (or 256) contiguous bytes with the same 5
// load instructions per matrix.  (Measured on GB300: the tiles cut k_lines
// 0.44 -> 0.27 ms and k_fwd 2.95 -> 2.63 ms against an 80-byte stride; the
// 72-byte tile moves 10% fewer bytes than a padded 80-byte one.)  FP64: 18
// reals as 9 double2 per (plane, site), contiguous (144 B).
template <typename T>
struct MatAoS;
template <>
struct MatAoS<float> {
    float4* __restrict__ p;
    int64_t V;
    int nk = 0;  // planes, checked when > 0 (bounds-checked build)
    __device__ __forceinline__ bool ok(int64_t s, int k) const {
        return FLUE_INB(s >= 0 && s < V && k >= 0 && (nk == 0 || k < nk));
    }
    __device__ __forceinline__ int64_t tile0(int64_t s, int k) const {
        return ((int64_t)k * ((V + 31) >> 5) + (s >> 5)) * 144;
    }
    __device__ __forceinline__ static M3<float> unpack(const float4* q, const float2* r) {
        M3<float> m;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 v = q[32 * j];
            m.r[2 * j] = v.x;
            m.i[2 * j] = v.y;
            m.r[2 * j + 1] = v.z;
            m.i[2 * j + 1] = v.w;
        }
        const float2 v = *r;
        m.r[8] = v.x;
        m.i[8] = v.y;
        return m;
    }
    __device__ __forceinline__ M3<float> load(int64_t s, int k) const {
        if (!ok(s, k)) return m_zero<float>();
        const int64_t t = tile0(s, k);
        return unpack(p + t + (s & 31), reinterpret_cast<const float2*>(p + t + 128) + (s & 31));
    }
    __device__ __forceinline__ void store(int64_t s, int k, const M3<float>& m) const {
        if (!ok(s, k)) return;
        const int64_t t = tile0(s, k);
        float4* q = p + t + (s & 31);
#pragma unroll
        for (int j = 0; j < 4; ++j) q[32 * j] = make_float4(m.r[2 * j], m.i[2 * j], m.r[2 * j + 1], m.i[2 * j + 1]);
        reinterpret_cast<float2*>(p + t + 128)[s & 31] = make_float2(m.r[8], m.i[8]);
    }
    // 32-bit form of the address arithmetic, for buffers of fewer than 2^31
    // float4 units (fits32): plane k starts k * pstride32() units in, the
    // tile of site s (s >> 5) * 144 units into its plane
    __device__ __forceinline__ uint32_t pstride32() const { return (uint32_t)((V + 31) >> 5) * 144u; }
    __device__ __forceinline__ uint32_t tile0_32(uint32_t s, int k) const {
        return (uint32_t)k * pstride32() + (s >> 5) * 144u;
    }
    // the float4 units 0..3 (at +32 u) and the float2 unit of site s
    __device__ __forceinline__ const float4* unit0_32(uint32_t s, int k) const { return p + tile0_32(s, k) + (s & 31u); }
    __device__ __forceinline__ const float2* unit4_32(uint32_t s, int k) const {
        return reinterpret_cast<const float2*>(p + tile0_32(s, k) + 128u) + (s & 31u);
    }
    __device__ __forceinline__ M3<float> load32(uint32_t s, int k) const {
        if (!ok((int64_t)s, k)) return m_zero<float>();
        const uint32_t t = tile0_32(s, k);
        return unpack(p + t + (s & 31u), reinterpret_cast<const float2*>(p + t + 128u) + (s & 31u));
    }
    static bool fits32(int64_t V, int64_t nk) { return (uint64_t)nk * (uint64_t)((V + 31) >> 5) * 144u < (1ull << 31); }
    static constexpr size_t bytes_per_matrix = 72;
    // bytes of nk planes over V sites (V rounded up to whole tiles)
    static size_t bytes(int64_t V, int64_t nk) { return (size_t)nk * (size_t)((V + 31) >> 5) * 2304; }
};
template <>
struct MatAoS<double> {
    double2* __restrict__ p;
    int64_t V;
    int nk = 0;  // planes, checked when > 0 (bounds-checked build)
    __device__ __forceinline__ bool ok(int64_t s, int k) const {
        return FLUE_INB(s >= 0 && s < V && k >= 0 && (nk == 0 || k < nk));
    }
    __device__ __forceinline__ M3<double> load(int64_t s, int k) const {
        if (!ok(s, k)) return m_zero<double>();
        const double2* q = p + ((int64_t)k * V + s) * 9;
        M3<double> m;
#pragma unroll
        for (int e = 0; e < 9; ++e) {
            const double2 v = q[e];
            m.r[e] = v.x;
            m.i[e] = v.y;
        }
        return m;
    }
    __device__ __forceinline__ void store(int64_t s, int k, const M3<double>& m) const {
        if (!ok(s, k)) return;
        double2* q = p + ((int64_t)k * V + s) * 9;
#pragma unroll
        for (int e = 0; e < 9; ++e) q[e] = make_double2(m.r[e], m.i[e]);
    }
    // 32-bit form (fits32): matrix (k, s) at (k * V + s) * 9 double2 units
    __device__ __forceinline__ M3<double> load32(uint32_t s, int k) const {
        if (!ok((int64_t)s, k)) return m_zero<double>();
        const double2* q = p + ((uint32_t)k * (uint32_t)V + s) * 9u;
        M3<double> m;
#pragma unroll
        for (int e = 0; e < 9; ++e) {
            const double2 v = q[e];
            m.r[e] = v.x;
            m.i[e] = v.y;
        }
        return m;
    }
    static bool fits32(int64_t V, int64_t nk) { return (uint64_t)nk * (uint64_t)V * 9u < (1ull << 31); }
    static constexpr size_t bytes_per_matrix = 144;
    static size_t bytes(int64_t V, int64_t nk) { return (size_t)nk * (size_t)V * 144; }
};

// Anti-Hermitian matrix per (plane k, site s), contiguous: Im F00, Im F11,
// Im F22, F01, F02, F12 (re, im) -- 9 reals padded to 12 (FP32, 3 float4) or
// 10 (FP64, 5 double2).
template <typename T>
__device__ __forceinline__ M3<T> ah_expand(const T v[9]) {
    M3<T> m;
    m.r[0] = m.r[4] = m.r[8] = T(0);
    m.i[0] = v[0];
    m.i[4] = v[1];
    m.i[8] = v[2];
    m.r[1] = v[3];
    m.i[1] = v[4];
    m.r[3] = -v[3];
    m.i[3] = v[4];
    m.r[2] = v[5];
    m.i[2] = v[6];
    m.r[6] = -v[5];
    m.i[6] = v[6];
    m.r[5] = v[7];
    m.i[5] = v[8];
    m.r[7] = -v[7];
    m.i[7] = v[8];
    return m;
}
// Products with an anti-Hermitian K given as its 9 packed reals (Im K00,
// Im K11, Im K22, K01, K02, K12): the real diagonal is zero, so each output
// element costs 10 FMA instead of 12.
template <typename T>
__device__ __forceinline__ T ahr(const T v[9], int a, int c) {  // Re K_ac
    return (a == c) ? T(0)
           : (a == 0 && c == 1) ? v[3]
           : (a == 0 && c == 2) ? v[5]
           : (a == 1 && c == 2) ? v[7]
           : (a == 1 && c == 0) ? -v[3]
           : (a == 2 && c == 0) ? -v[5]
                                : -v[7];
}
template <typename T>
__device__ __forceinline__ T ahi(const T v[9], int a, int c) {  // Im K_ac
    return (a == c) ? v[a] : ((a + c) == 1) ? v[4] : ((a + c) == 2) ? v[6] : v[8];
}
// C += K op(X), op = dagger when DX
template <bool DX = false, typename T>
__device__ __forceinline__ void mac_kx(M3<T>& C, const T k[9], const M3<T>& X) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            T re = C.r[3 * a + b], im = C.i[3 * a + b];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T xr = DX ? X.r[3 * b + c] : X.r[3 * c + b];
                const T xi = DX ? -X.i[3 * b + c] : X.i[3 * c + b];
                const T ki = ahi(k, a, c);
                if (a != c) {
                    const T kr = ahr(k, a, c);
                    re = fma(kr, xr, re);
                    im = fma(kr, xi, im);
                }
                re = fma(-ki, xi, re);
                im = fma(ki, xr, im);
            }
            C.r[3 * a + b] = re;
            C.i[3 * a + b] = im;
        }
}
// C += op(X) K, op = dagger when DX
template <bool DX = false, typename T>
__device__ __forceinline__ void mac_xk(M3<T>& C, const M3<T>& X, const T k[9]) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            T re = C.r[3 * a + b], im = C.i[3 * a + b];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T xr = DX ? X.r[3 * c + a] : X.r[3 * a + c];
                const T xi = DX ? -X.i[3 * c + a] : X.i[3 * a + c];
                const T ki = ahi(k, c, b);
                if (c != b) {
                    const T kr = ahr(k, c, b);
                    re = fma(xr, kr, re);
                    im = fma(xi, kr, im);
                }
                re = fma(-xi, ki, re);
                im = fma(xr, ki, im);
            }
            C.r[3 * a + b] = re;
            C.i[3 * a + b] = im;
        }
}

template <typename T>
struct AHAoS;
template <>
struct AHAoS<float> {
    // 9 reals padded to 3 float4 units, tiled by 32 sites as MatAoS<float>:
    // unit u of site s of plane k at ((k * T + s / 32) * 3 + u) * 32 + s % 32
    float4* __restrict__ p;
    int64_t V;
    int nk = 0;  // planes, checked when > 0 (bounds-checked build)
    __device__ __forceinline__ bool ok(int64_t s, int k) const {
        return FLUE_INB(s >= 0 && s < V && k >= 0 && (nk == 0 || k < nk));
    }
    __device__ __forceinline__ const float4* unit0(int64_t s, int k) const {
        return p + (((int64_t)k * ((V + 31) >> 5) + (s >> 5)) * 3) * 32 + (s & 31);
    }
    __device__ __forceinline__ void load_packed(int64_t s, int k, float v[9]) const {
        if (!ok(s, k)) {
            for (int e = 0; e < 9; ++e) v[e] = 0;
            return;
        }
        const float4* q = unit0(s, k);
        const float4 a = q[0], b = q[32], c = q[64];
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w;
        v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
        v[8] = c.x;
    }
    // 32-bit form (fits32)
    __device__ __forceinline__ void load_packed32(uint32_t s, int k, float v[9]) const {
        if (!ok((int64_t)s, k)) {
            for (int e = 0; e < 9; ++e) v[e] = 0;
            return;
        }
        const float4* q = p + ((uint32_t)k * ((uint32_t)((V + 31) >> 5) * 96u) + (s >> 5) * 96u + (s & 31u));
        const float4 a = q[0], b = q[32], c = q[64];
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w;
        v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
        v[8] = c.x;
    }
    static bool fits32(int64_t V, int64_t nk) { return (uint64_t)nk * (uint64_t)((V + 31) >> 5) * 96u < (1ull << 31); }
    __device__ __forceinline__ M3<float> load(int64_t s, int k) const {
        if (!ok(s, k)) return m_zero<float>();
        float v[9];
        load_packed(s, k, v);
        return ah_expand<float>(v);
    }
    __device__ __forceinline__ void store(int64_t s, int k, const M3<float>& m) const {
        if (!ok(s, k)) return;
        float4* q = const_cast<float4*>(unit0(s, k));
        q[0] = make_float4(m.i[0], m.i[4], m.i[8], m.r[1]);
        q[32] = make_float4(m.i[1], m.r[2], m.i[2], m.r[5]);
        q[64] = make_float4(m.i[5], 0.f, 0.f, 0.f);
    }
    static constexpr size_t bytes_per_matrix = 48;
    static size_t bytes(int64_t V, int64_t nk) { return (size_t)nk * (size_t)((V + 31) & ~(int64_t)31) * 48; }
};
template <>
struct AHAoS<double> {
    double2* __restrict__ p;
    int64_t V;
    int nk = 0;  // planes, checked when > 0 (bounds-checked build)
    __device__ __forceinline__ bool ok(int64_t s, int k) const {
        return FLUE_INB(s >= 0 && s < V && k >= 0 && (nk == 0 || k < nk));
    }
    __device__ __forceinline__ void load_packed(int64_t s, int k, double v[9]) const {
        if (!ok(s, k)) {
            for (int e = 0; e < 9; ++e) v[e] = 0;
            return;
        }
        const double2* q = p + ((int64_t)k * V + s) * 5;
        const double2 a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
        v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y, v[4] = c.x;
        v[5] = c.y, v[6] = d.x, v[7] = d.y, v[8] = e.x;
    }
    // 32-bit form (fits32)
    __device__ __forceinline__ void load_packed32(uint32_t s, int k, double v[9]) const {
        if (!ok((int64_t)s, k)) {
            for (int e = 0; e < 9; ++e) v[e] = 0;
            return;
        }
        const double2* q = p + ((uint32_t)k * (uint32_t)V + s) * 5u;
        const double2 a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
        v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y, v[4] = c.x;
        v[5] = c.y, v[6] = d.x, v[7] = d.y, v[8] = e.x;
    }
    static bool fits32(int64_t V, int64_t nk) { return (uint64_t)nk * (uint64_t)V * 5u < (1ull << 31); }
    __device__ __forceinline__ M3<double> load(int64_t s, int k) const {
        if (!ok(s, k)) return m_zero<double>();
        const double2* q = p + ((int64_t)k * V + s) * 5;
        const double2 a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
        const double v[9] = {a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x};
        return ah_expand<double>(v);
    }
    __device__ __forceinline__ void store(int64_t s, int k, const M3<double>& m) const {
        if (!ok(s, k)) return;
        double2* q = p + ((int64_t)k * V + s) * 5;
        q[0] = make_double2(m.i[0], m.i[4]);
        q[1] = make_double2(m.i[8], m.r[1]);
        q[2] = make_double2(m.i[1], m.r[2]);
        q[3] = make_double2(m.i[2], m.r[5]);
        q[4] = make_double2(m.i[5], 0.0);
    }
    static constexpr size_t bytes_per_matrix = 80;
    static size_t bytes(int64_t V, int64_t nk) { return (size_t)nk * (size_t)V * 80; }
};

// Anti-Hermitian matrices stored as 9 reals per site: Im F00, Im F11, Im F22,
// F01 (re, im), F02 (re, im), F12 (re, im) at base[(k*9 + e)*V + s].
template <typename T>
struct AHPlanes {
    T* __restrict__ p;
    int64_t V;
    __device__ __forceinline__ M3<T> load(int64_t s, int k) const {
        if (!FLUE_INB(s >= 0 && s < V && k >= 0)) return m_zero<T>();
        const T* q = p + (int64_t)k * 9 * V + s;
        T v[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) v[e] = q[e * V];
        M3<T> m;
        m.r[0] = m.r[4] = m.r[8] = T(0);
        m.i[0] = v[0];
        m.i[4] = v[1];
        m.i[8] = v[2];
        m.r[1] = v[3];
        m.i[1] = v[4];
        m.r[3] = -v[3];
        m.i[3] = v[4];
        m.r[2] = v[5];
        m.i[2] = v[6];
        m.r[6] = -v[5];
        m.i[6] = v[6];
        m.r[5] = v[7];
        m.i[5] = v[8];
        m.r[7] = -v[7];
        m.i[7] = v[8];
        return m;
    }
    __device__ __forceinline__ void store(int64_t s, int k, const M3<T>& m) const {
        if (!FLUE_INB(s >= 0 && s < V && k >= 0)) return;
        T* q = p + (int64_t)k * 9 * V + s;
        q[0] = m.i[0];
        q[V] = m.i[4];
        q[2 * V] = m.i[8];
        q[3 * V] = m.r[1];
        q[4 * V] = m.i[1];
        q[5 * V] = m.r[2];
        q[6 * V] = m.i[2];
        q[7 * V] = m.r[5];
        q[8 * V] = m.i[5];
    }
};

// Output in the reference layout (NT,NX,NY,NZ,[4,]3,3): element (s, slot, a, b)
// at s + V*(slot + nslot*(a + 3b)).  The caller picks transpose on store.
template <typename T>
struct RefOut {
    using C2 = typename V2<T>::type;
    C2* __restrict__ p;
    int64_t V;
    int nslot;
    // T-slab output (nts > 0): site s of a sub-lattice with nts time slices
    // goes to site t0 + s % nts + ntf * (s / nts) of the full lattice, whose
    // time extent is ntf and volume V.  nts = 0: site s is site s.
    int nts = 0, ntf = 0, t0 = 0;
    // complex128 destination of an FP32 computation (p unused when set): the
    // gradient of a complex128 field computed in FP32 is written back in the
    // field's own dtype
    double2* __restrict__ pd = nullptr;
    __device__ __forceinline__ void store(int64_t s, int slot, const M3<T>& m) const {
        const int64_t sf = nts ? (int64_t)t0 + s % nts + (int64_t)ntf * (s / nts) : s;
        if (!FLUE_INB(sf >= 0 && sf < V && slot >= 0 && slot < nslot)) return;
        const int64_t st = V * nslot;
        if (pd) {
            double2* q = pd + sf + V * slot;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) q[st * (a + 3 * b)] = make_double2(m.r[3 * a + b], m.i[3 * a + b]);
            return;
        }
        C2* q = p + sf + V * slot;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                C2 v;
                v.x = m.r[3 * a + b];
                v.y = m.i[3 * a + b];
                q[st * (a + 3 * b)] = v;
            }
    }
};

// ---------------------------------------------------------------------------
// Geometry
// ---------------------------------------------------------------------------
struct Geom {
    int n[4];       // extents: NT, NX, NY, NZ
    int64_t st[4];  // site strides: 1, NT, NT*NX, NT*NX*NY
    int64_t V;
};

__host__ __device__ inline Geom make_geom(int nt, int nx, int ny, int nz) {
    Geom g;
    g.n[0] = nt;
    g.n[1] = nx;
    g.n[2] = ny;
    g.n[3] = nz;
    g.st[0] = 1;
    g.st[1] = nt;
    g.st[2] = (int64_t)nt * nx;
    g.st[3] = (int64_t)nt * nx * ny;
    g.V = (int64_t)nt * nx * ny * nz;
    return g;
}

__device__ __forceinline__ void site_coords(const Geom& g, int64_t s, int c[4]) {
    int64_t r = s;
    c[0] = (int)(r % g.n[0]);
    r /= g.n[0];
    c[1] = (int)(r % g.n[1]);
    r /= g.n[1];
    c[2] = (int)(r % g.n[2]);
    c[3] = (int)(r / g.n[2]);
}

// Site offset of a displacement by k (any sign, |k| <= 4*n) along mu from a
// site whose mu-coordinate is cmu, with periodic wrap.
__device__ __forceinline__ int64_t disp(const Geom& g, int mu, int cmu, int k) {
    const int n = g.n[mu];
    int t = (cmu + k) % n;
    if (t < 0) t += n;
    return (int64_t)(t - cmu) * g.st[mu];
}

// ---------------------------------------------------------------------------
// Deterministic reductions: every block writes one FP64 partial per output
// slot; a single-block finisher sums them in index order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum (blockDim.x a multiple of 32, <= 1024); result valid in
// thread 0.  `sh` must hold 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = lane < nw ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

}  // namespace flue
