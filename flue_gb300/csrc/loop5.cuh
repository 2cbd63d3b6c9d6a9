// loop5.cuh -- device building blocks of the 5-loop field strength shared by
// the energy / force pipeline (force.cu) and the persistent ensemble kernel
// (ensemble.cu): the shape table, plane descriptors, the straight lines
// L^a_d(y) = U_d(y) U_d(y+d) ... U_d(y+(a-1)d) and the leaf sum Q of one
// site and plane built from them (src/wloops.F90:201-432).
#pragma once
#include "flue_common.cuh"

namespace flue {

// 5-loop coefficients, src/wloops.F90:219-224 (k5 = 1/180).
constexpr double K5c = 1.0 / 180.0;
constexpr double K1c = (19.0 / 9.0) - 55.0 * K5c;
constexpr double K2c = (1.0 / 36.0) - 16.0 * K5c;
constexpr double K3c = 64.0 * K5c - (32.0 / 45.0);
constexpr double K4c = (1.0 / 15.0) - 6.0 * K5c;

struct Shape {
    int a, b;
    double c;
};
// kind 1: 5-loop (weights of :327, :341, :358, :382, :405); kind 0: clover.
static __constant__ Shape c_shapes5[7] = {{1, 1, K1c},       {2, 2, K2c},       {3, 3, K5c},      {1, 2, 0.5 * K3c},
                                          {2, 1, 0.5 * K3c}, {1, 3, 0.5 * K4c}, {3, 1, 0.5 * K4c}};
static __constant__ Shape c_shapes1[1] = {{1, 1, 1.0}};

// The other extent w and the weight of every 5-loop shape that has a side of
// length len (shapes (len, w) and (w, len) carry the same coefficient,
// src/wloops.F90:219-224, :327-405): row len - 1, w = 0 ends the row.
static __constant__ int c_lw_w[3][3] = {{1, 2, 3}, {2, 1, 0}, {3, 1, 0}};
static __constant__ double c_lw_c[3][3] = {{K1c, 0.5 * K3c, 0.5 * K4c}, {K2c, 0.5 * K3c, 0.0}, {K5c, 0.5 * K4c, 0.0}};
// the same weights rounded to FP32 once (no FP64 -> FP32 conversion in the
// FP32 kernel's inner loop)
static __constant__ float c_lw_cf[3][3] = {{(float)K1c, (float)(0.5 * K3c), (float)(0.5 * K4c)},
                                    {(float)K2c, (float)(0.5 * K3c), 0.f},
                                    {(float)K5c, (float)(0.5 * K4c), 0.f}};
template <typename T>
__device__ __forceinline__ T lw_coef(int len, int k);
template <>
__device__ __forceinline__ float lw_coef<float>(int len, int k) {
    return c_lw_cf[len - 1][k];
}
template <>
__device__ __forceinline__ double lw_coef<double>(int len, int k) {
    return c_lw_c[len - 1][k];
}

// Planes and direction slots of one energy evaluation.
struct PlaneArg {
    int np;
    int mu[6], nu[6];
    int nd;
    int slot[4];  // direction -> slot, -1 if unused
    int dir[4];   // slot -> direction
};

// Reads of PlaneArg with a runtime index, written as unrolled selects so that
// the kernel-parameter struct is never copied to local memory.
template <int N>
__device__ __forceinline__ int sel(const int (&a)[N], int i) {
    int r = a[0];
#pragma unroll
    for (int k = 1; k < N; ++k)
        if (k == i) r = a[k];
    return r;
}

__device__ __forceinline__ int wrapd(int c, int k, int n) {
    int t = c + k;
    if (n > 3) {  // every stencil offset is within +-3: one conditional wrap
        t += (t < 0) ? n : 0;
        t -= (t >= n) ? n : 0;
    } else {
        while (t < 0) t += n;
        while (t >= n) t -= n;
    }
    return t - c;
}


// Per-thread view of one plane (mu,nu) around the thread's site: every
// coordinate the stencil needs is kept in scalars (no runtime-indexed
// arrays, so nothing lands in local memory).
template <typename T>
struct Ctx {
    MatAoS<T> lines;  // 3 per slot: L^1 (U expanded), L^2, L^3
    int64_t s;
    int cm, cn, nm, nn;  // coordinates and extents along mu, nu
    int64_t stm, stn;    // site strides along mu, nu
    int kmu, knu;        // first line plane of the mu / nu slot (3 * slot)
};

template <typename T>
__device__ __forceinline__ Ctx<T> make_ctx(const MatAoS<T>& lines, const Geom& g, int64_t s, const int c[4], int mu,
                                           int nu, int smu, int snu) {
    Ctx<T> cx;
    cx.lines = lines;
    cx.s = s;
    // select without runtime indexing of c[] / g.n[] / g.st[]
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        if (d == mu) {
            cx.cm = c[d];
            cx.nm = g.n[d];
            cx.stm = g.st[d];
        }
        if (d == nu) {
            cx.cn = c[d];
            cx.nn = g.n[d];
            cx.stn = g.st[d];
        }
    }
    cx.kmu = 3 * smu;
    cx.knu = 3 * snu;
    return cx;
}


// Loads through 32-bit (I = uint32_t) or 64-bit (I = int64_t) address
// arithmetic; the 32-bit form is used when every buffer the kernel indexes
// has fewer than 2^31 vector units (MatAoS / AHAoS fits32).
template <typename T>
__device__ __forceinline__ M3<T> ldm(const MatAoS<T>& m, uint32_t s, int k) {
    return m.load32(s, k);
}
template <typename T>
__device__ __forceinline__ M3<T> ldm(const MatAoS<T>& m, int64_t s, int k) {
    return m.load(s, k);
}
template <typename T>
__device__ __forceinline__ void ldk(const AHAoS<T>& m, uint32_t s, int k, T v[9]) {
    m.load_packed32(s, k, v);
}
template <typename T>
__device__ __forceinline__ void ldk(const AHAoS<T>& m, int64_t s, int k, T v[9]) {
    m.load_packed(s, k, v);
}

// Lines of one site and direction slot: L^1_d(s) = U_d (expanded to 18
// reals), L^2_d(s) = U_d(s) U_d(s+d), L^3_d(s) = L^2_d(s) U_d(s+2d).  Site s
// is one of geometry g; the links are read from a field of geometry gs at
// time offset t0 (gs = g, t0 = 0 for a whole lattice; a time slab of a larger
// field otherwise -- the lines never step in time then).
template <class L, typename T>
__device__ __forceinline__ void line_site(const L& U, const Geom& g, const Geom& gs, int t0, const PlaneArg& pa,
                                          const MatAoS<T>& lines, int64_t s, int slot) {
    const int d = sel(pa.dir, slot);
    int c[4];
    site_coords(g, s, c);
    int cd = 0, nd = 1;
    int64_t sd = 1;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k == d) cd = c[k], nd = g.n[k], sd = gs.st[k];
    const int64_t u = (int64_t)(t0 + c[0]) + c[1] * gs.st[1] + c[2] * gs.st[2] + c[3] * gs.st[3];
    const int64_t s1 = u + (int64_t)wrapd(cd, 1, nd) * sd;
    const int64_t s2 = u + (int64_t)wrapd(cd, 2, nd) * sd;
    const M3<T> u0 = U.load(u, d);
    const M3<T> l2 = mul(u0, U.load(s1, d));
    lines.store(s, 3 * slot, u0);
    lines.store(s, 3 * slot + 1, l2);
    const M3<T> l3 = mul(l2, U.load(s2, d));
    lines.store(s, 3 * slot + 2, l3);
}

// Q = sum over shapes and quadrants of the weighted leaves at site s (with
// coordinates c) in plane p of pa; kind 1: the 5-loop shapes, 0: the clover.
// 5-loop Q with the leaves of each quadrant grouped by the extent of their
// end line.  With L(i, j) the line at offset (i mu + j nu) (mu-lines of
// length a, nu-lines of length b):
//   TR = Lm(0,0) [Ln(a,0) Lm(0,b)^+] Ln(0,0)^+      BL = Lm(-a,0)^+ [Ln(-a,-b)^+ Lm(-a,-b)] Ln(0,-b)
//   TL = Ln(0,0) [Lm(-a,b)^+ Ln(-a,0)^+] Lm(-a,0)   BR = Ln(0,-b)^+ [Lm(0,-b) Ln(a,-b)] Lm(0,0)^+
// Lm(0,0) and Lm(-a,0) depend on a only, Ln(0,0) and Ln(0,-b) on b only, so
//   sum_ab c_ab TR = sum_a Lm(0,0) [sum_b c_ab (Ln(a,0) Lm(0,b)^+) Ln(0,0)^+]
// and likewise BL (grouped by a) and TL, BR (grouped by b): 8 products per
// shape and 2 per group, 68 per plane-site against 84 for the leaves one by
// one.  The groups are the rows of c_lw_w / c_lw_c (a side of length len,
// the other extent w).
template <typename T, typename I>
__device__ __forceinline__ M3<T> fwd_q5(const MatAoS<T>& lines, const Ctx<T>& cx) {
    const int s0 = (int)cx.s, stm = (int)cx.stm, stn = (int)cx.stn;
    auto ld = [&](int site, int k) { return ldm(lines, (I)site, k); };
    M3<T> q = m_zero<T>();
    // TR and BL, grouped by a
#pragma unroll 1
    for (int a = 1; a <= 3; ++a) {
        const int km = cx.kmu + a - 1;
        const int mM = wrapd(cx.cm, -a, cx.nm) * stm, mP = wrapd(cx.cm, a, cx.nm) * stm;
        M3<T> itr = m_zero<T>(), ibl = m_zero<T>();
        const int nb = a == 1 ? 3 : 2;
#pragma unroll 1
        for (int j = 0; j < nb; ++j) {
            const int b = c_lw_w[a - 1][j];
            const T cf = lw_coef<T>(a, j);
            const int kn = cx.knu + b - 1;
            const int nM = wrapd(cx.cn, -b, cx.nn) * stn, nP = wrapd(cx.cn, b, cx.nn) * stn;
            M3<T> t = mm<false, true>(ld(s0 + mP, kn), ld(s0 + nP, km));
            t = mm<false, true>(t, ld(s0, kn));
            m_axpy(itr, cf, t);
            t = mm<true, false>(ld(s0 + mM + nM, kn), ld(s0 + mM + nM, km));
            t = mm<false, false>(t, ld(s0 + nM, kn));
            m_axpy(ibl, cf, t);
        }
        mac<false, false>(q, ld(s0, km), itr);
        mac<true, false>(q, ld(s0 + mM, km), ibl);
    }
    // TL and BR, grouped by b
#pragma unroll 1
    for (int b = 1; b <= 3; ++b) {
        const int kn = cx.knu + b - 1;
        const int nM = wrapd(cx.cn, -b, cx.nn) * stn;
        M3<T> itl = m_zero<T>(), ibr = m_zero<T>();
        const int na = b == 1 ? 3 : 2;
#pragma unroll 1
        for (int j = 0; j < na; ++j) {
            const int a = c_lw_w[b - 1][j];
            const T cf = lw_coef<T>(b, j);
            const int km = cx.kmu + a - 1;
            const int mM = wrapd(cx.cm, -a, cx.nm) * stm, mP = wrapd(cx.cm, a, cx.nm) * stm;
            const int nP = wrapd(cx.cn, b, cx.nn) * stn;
            M3<T> t = mm<true, true>(ld(s0 + mM + nP, km), ld(s0 + mM, kn));
            t = mm<false, false>(t, ld(s0 + mM, km));
            m_axpy(itl, cf, t);
            t = mm<false, false>(ld(s0 + nM, km), ld(s0 + mP + nM, kn));
            t = mm<false, true>(t, ld(s0, km));
            m_axpy(ibr, cf, t);
        }
        mac<false, false>(q, ld(s0, kn), itl);
        mac<true, false>(q, ld(s0 + nM, kn), ibr);
    }
    return q;
}

template <typename T, typename I>
__device__ __forceinline__ M3<T> fwd_q(const Geom& g, const PlaneArg& pa, int kind, const MatAoS<T>& lines, int64_t s,
                                       const int c[4], int p) {
    const int pmu = sel(pa.mu, p), pnu = sel(pa.nu, p);
    // FP64 (bound by the FP64 pipe) takes the grouped form, 19% fewer
    // products: 96-field ensemble 3.46 -> 3.09 s per evaluation on GB300.
    // FP32 (issue- and latency-bound at 12 warps per SM) keeps the leaves one
    // by one: the grouped form's extra line loads and shorter independent
    // chains made its forward slower, 2.56 -> 2.72 ms at 32^3x64.
    if constexpr (sizeof(T) == 8) {
        if (kind == 1) {
            const Ctx<T> cx5 = make_ctx(lines, g, s, c, pmu, pnu, sel(pa.slot, pmu), sel(pa.slot, pnu));
            return fwd_q5<T, I>(lines, cx5);
        }
    }
    const Ctx<T> cx = make_ctx(lines, g, s, c, pmu, pnu, sel(pa.slot, pmu), sel(pa.slot, pnu));
    const Shape* shp = kind == 1 ? c_shapes5 : c_shapes1;
    const int nsh = kind == 1 ? 7 : 1;
    M3<T> q = m_zero<T>();
    // Per shape the four quadrant leaves, with their dagger patterns fixed
    // at compile time (lines are loaded undaggered; L(i,j) = line at
    // offset (i mu + j nu)):
    //   TR = Lm(0,0) Ln(a,0) Lm(0,b)^+ Ln(0,0)^+
    //   TL = Ln(0,0) Lm(-a,b)^+ Ln(-a,0)^+ Lm(-a,0)
    //   BL = Lm(-a,0)^+ Ln(-a,-b)^+ Lm(-a,-b) Ln(0,-b)
    //   BR = Ln(0,-b)^+ Lm(0,-b) Ln(a,-b) Lm(0,0)^+
    // Lm(0,0), Ln(0,0), Lm(-a,0), Ln(0,-b) serve two leaves each.
#pragma unroll 1
    for (int k = 0; k < nsh; ++k) {
        const int a = shp[k].a, b = shp[k].b;
        const int km = cx.kmu + a - 1, kn = cx.knu + b - 1;
        // the 3 x 3 sites (i, j) in {-a, 0, a} x {-b, 0, b} the leaves use
        // (site offsets within the lattice are 32-bit; the address
        // arithmetic is 32-bit too when I = uint32_t)
        const int s0 = (int)cx.s, stm = (int)cx.stm, stn = (int)cx.stn;
        const int mM = wrapd(cx.cm, -a, cx.nm) * stm, mP = wrapd(cx.cm, a, cx.nm) * stm;
        const int nM = wrapd(cx.cn, -b, cx.nn) * stn, nP = wrapd(cx.cn, b, cx.nn) * stn;
        auto ld = [&](int site, int k) { return ldm(lines, (I)site, k); };
        M3<T> w;
        {
            const M3<T> m00 = ld(s0, km);
            const M3<T> n00 = ld(s0, kn);
            M3<T> t = mm<false, false>(m00, ld(s0 + mP, kn));
            t = mm<false, true>(t, ld(s0 + nP, km));
            w = mm<false, true>(t, n00);  // TR
            const M3<T> ma0 = ld(s0 + mM, km);
            t = mm<false, true>(n00, ld(s0 + mM + nP, km));
            t = mm<false, true>(t, ld(s0 + mM, kn));
            mac<false, false>(w, t, ma0);  // TL
            const M3<T> n0b = ld(s0 + nM, kn);
            t = mm<true, true>(ma0, ld(s0 + mM + nM, kn));
            t = mm<false, false>(t, ld(s0 + mM + nM, km));
            mac<false, false>(w, t, n0b);  // BL
            t = mm<true, false>(n0b, ld(s0 + nM, km));
            t = mm<false, false>(t, ld(s0 + mP + nM, kn));
            mac<false, true>(w, t, m00);  // BR
        }
        m_axpy(q, (T)shp[k].c, w);
    }
    return q;
}

}  // namespace flue
