// force.cu -- clover and 5-loop F_munu, the 5-loop energy / B^2 and its
// su(3) gradient, and the Wilson plaquette-action force.
//
// The 5-loop field strength (src/wloops.F90:201-432, hep-lat/0203008) at a
// site x and plane (mu,nu) is built from the 28 counter-clockwise leaves of
// the rectangles of shapes (a,b) in {(1,1),(2,2),(3,3),(1,2),(2,1),(1,3),(3,1)}
// (a links along mu, b along nu) that have x as a corner.  The reference walks
// every leaf link by link (208 link steps and 180 products per plane-site);
// here a leaf is the product of four straight "lines"
//     L^a_mu(y) = U_mu(y) U_mu(y+mu) ... U_mu(y+(a-1)mu),   a = 1,2,3,
// precomputed once per site (2 products per direction), so a leaf costs 3
// products (84 per plane-site).  Writing the rectangle anchored at y0 (its
// lower-left corner) as the sides
//     S1 = L^a_mu(y0),  S2 = L^b_nu(y0+a mu),  S3 = L^a_mu(y0+b nu)^+,  S4 = L^b_nu(y0)^+
// with corners K1..K4 at y0, y0+a mu, y0+a mu+b nu, y0+b nu, the leaf of x in
// quadrant q is the cyclic word S_q S_q+1 S_q+2 S_q+3 of the rectangle that
// has x as its corner q.  genericPath returns the transpose of every leaf
// (:56); the kernels work with untransposed leaves and transpose on output.
//
// Energy E = -1/V sum_x sum_planes Re Tr(F F) (B^2 for the three spatial
// planes (3,2),(2,4),(4,3) of magnetic, :502-506).  Reverse mode, written as
// gathers so that no atomics are needed and results are deterministic:
//   1. lines:   L^2, L^3 per direction                    (k_lines)
//   2. forward: Q, F = AH(Q)/4, E partials; F kept as the cotangent
//               dE/dQ = -F/(2V) (stored as 9 reals)        (k_fwd)
//   3. line cotangents: Lambda^a_d(y) with dE = Re Tr(dL Lambda), summed over
//      every rectangle side that is the line (y,d,a); each side collects the
//      four corner insertions K S S S + S K S S + S S K S + S S S K with a
//      Horner scheme (8 products)                          (k_linecot)
//   4. link cotangents N_d(z) from the line cotangents of the lines through
//      the link, then the su(3)-projected gradient G = -1/2 TA(U N) or the
//      Euclidean gradient N^+                              (k_linkcot)
#include <stdlib.h>

#include <mutex>

#include "flue_internal.h"
#include "loop5.cuh"

namespace flue {

// Traversal order of the site blocks of the stencil kernels.  The lattice is
// a sequence of rows (fixed y, z) of NT*NX sites.  When a row holds a whole
// number of blocks and NY, NZ are multiples of the tile, rows are visited in
// TILE x TILE (y,z) tiles, y fastest, so that the blocks in flight cover a
// compact neighbourhood and the +-3 halo they read is still in L2 (measured
// no faster on GB300: off by default).
#ifndef FLUE_TILE_YZ
#define FLUE_TILE_YZ 0
#endif
__device__ __forceinline__ int64_t site_block(int64_t b, const Geom& g, int bs) {
#if FLUE_TILE_YZ > 0
    const int T = FLUE_TILE_YZ;
    const int64_t rowlen = (int64_t)g.n[0] * g.n[1];
    if (rowlen % bs == 0 && g.n[2] % T == 0 && g.n[3] % T == 0) {
        const int64_t bpr = rowlen / bs;
        const int64_t in_row = b % bpr, row = b / bpr;
        const int64_t tile = row / (T * T), r = row % (T * T);
        const int64_t nty = g.n[2] / T;
        const int64_t y = (tile % nty) * T + r % T, z = (tile / nty) * T + r / T;
        return (y + (int64_t)g.n[2] * z) * bpr + in_row;
    }
#endif
    return b;
}

// Patch traversal of the stencil kernels: a block of `bs` threads covers tw
// consecutive time slices x a pm x pn patch of the plane (mu, nu) x po sites
// along the third spatial direction (tw * pm * pn * po = bs), so the warps of
// a block read overlapping neighbourhoods and share them in L1.  tw = 0: the
// linear order.  Valid for spatial planes with tw | NT, pm | N_mu, pn | N_nu,
// po | N_other (make_patch checks; otherwise it returns tw = 0).
struct PatchArg {
    int tw, pm, pn, po;
};

__device__ __forceinline__ int64_t patch_site(const Geom& g, const PatchArg& pt, int pmu, int pnu, int64_t r) {
    int nm = 1, nn = 1;
    int64_t stm = 0, stn = 0, sto = 0;
    const int od = 6 - pmu - pnu;
#pragma unroll
    for (int d = 1; d < 4; ++d) {
        if (d == pmu) nm = g.n[d], stm = g.st[d];
        if (d == pnu) nn = g.n[d], stn = g.st[d];
        if (d == od) sto = g.st[d];
    }
    const int ntc = g.n[0] / pt.tw, nbm = nm / pt.pm, nbn = nn / pt.pn;
    const int tc = (int)(r % ntc);
    r /= ntc;
    const int bi = (int)(r % nbm);
    r /= nbm;
    const int bj = (int)(r % nbn);
    const int bo = (int)(r / nbn);
    const int tid = threadIdx.x;
    const int tl = tid % pt.tw, pos = tid / pt.tw;
    const int im = pos % pt.pm, in = (pos / pt.pm) % pt.pn, io = pos / (pt.pm * pt.pn);
    return (int64_t)tc * pt.tw + tl + (int64_t)(bi * pt.pm + im) * stm + (int64_t)(bj * pt.pn + in) * stn +
           (int64_t)(bo * pt.po + io) * sto;
}

#ifndef FLUE_PATCH_MIN_TW
#define FLUE_PATCH_MIN_TW 8
#endif
static PatchArg make_patch(const Geom& g, const PlaneArg& pa, int bs) {
    PatchArg pt{0, 1, 1, 1};
    int tw = 1;
    while (tw < 32 && g.n[0] % (2 * tw) == 0 && tw * 2 <= bs) tw *= 2;
    const int P = bs / tw;
    int pm = 1;
    while (pm < 4 && pm * pm * 4 <= P) pm *= 2;  // pm = pn <= 4
    const int po = P / (pm * pm);
    for (int q = 0; q < pa.np; ++q) {
        const int mu = pa.mu[q], nu = pa.nu[q], od = 6 - mu - nu;
        if (mu <= 0 || nu <= 0 || g.n[mu] % pm || g.n[nu] % pm || g.n[od] % po) return pt;
    }
    // warps keep runs of >= FLUE_PATCH_MIN_TW consecutive sites (measured at
    // 32^3x64 in 4-slice slabs, tiled intermediates: minimum 4 -> 10.74 ms a
    // step, 8 -> 10.50 ms)
    if (tw * pm * pm * po != bs || tw < FLUE_PATCH_MIN_TW) return pt;
    pt.tw = tw;
    pt.pm = pt.pn = pm;
    pt.po = po;
    return pt;
}

// ---------------------------------------------------------------------------
// 1. lines: L^1_d(y) = U_d(y) (expanded to 18 reals), L^2_d(y) = U_d(y) U_d(y+d),
//    L^3_d(y) = L^2_d(y) U_d(y+2d).  Sites are those of geometry g; the links
//    are read from a field of geometry gs at time offset t0 (gs = g, t0 = 0
//    for a whole lattice; a time slab of a larger field otherwise -- the lines
//    never step in time then).
// ---------------------------------------------------------------------------
template <class L, typename T>
__global__ void k_lines(L U, Geom g, Geom gs, int t0, PlaneArg pa, MatAoS<T> lines) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.V) return;
    line_site<L, T>(U, g, gs, t0, pa, lines, s, (int)blockIdx.y);
}

// ---------------------------------------------------------------------------
// 2. forward: one thread per (site, plane)
// ---------------------------------------------------------------------------
// block size and minimum resident blocks per SM (register budget) of the
// forward and line-cotangent kernels; overridable at build time
#ifndef FLUE_FWD_BS
#define FLUE_FWD_BS 128
#endif
// patch traversal of the forward (PatchArg): 32^3x64 one pass 3.26 -> 2.95 ms;
// inside 4-slice time slabs it is not used (make_patch)
#ifndef FLUE_FWD_PATCH
#define FLUE_FWD_PATCH 1
#endif
#ifndef FLUE_FWD_MINB
#define FLUE_FWD_MINB 3
#endif
#ifndef FLUE_COT_BS
#define FLUE_COT_BS 128
#endif
#ifndef FLUE_COT_MINB
#define FLUE_COT_MINB 4
#endif
// the register caps apply to the FP32 kernels; the FP64 ones keep every
// register they need (they are bound by the FP64 pipe, not by latency)
template <typename T>
struct MinBlocks {
    static constexpr int fwd = 1, cot = 1;
};
template <>
struct MinBlocks<float> {
    static constexpr int fwd = FLUE_FWD_MINB, cot = FLUE_COT_MINB;
};
constexpr int FWD_BS = FLUE_FWD_BS;

template <typename T, typename I>
__global__ void __launch_bounds__(FWD_BS, MinBlocks<T>::fwd)
    k_fwd(Geom g, PlaneArg pa, int kind, PatchArg pt, MatAoS<T> lines, AHAoS<T> kout, RefOut<T> fout, double* part) {
    __shared__ double sh[32];
    // planes of the same site block run in adjacent blocks (L2 reuse)
    const int p = blockIdx.x % pa.np;
    const int pmu = sel(pa.mu, p), pnu = sel(pa.nu, p);
    const int64_t s = pt.tw ? patch_site(g, pt, pmu, pnu, blockIdx.x / pa.np)
                            : site_block(blockIdx.x / pa.np, g, blockDim.x) * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (s < g.V) {
        int c[4];
        site_coords(g, s, c);
        const M3<T> q = fwd_q<T, I>(g, pa, kind, lines, s, c, p);
        const M3<T> f = ah_quarter(q);
        e = -(double)retr_mm<false, false>(f, f);
        if (kout.p) kout.store(s, p, f);
        if (fout.p) fout.store(s, 0, transp(f));
    }
    if (part) {
        const double r = block_sum(e, sh);
        if (threadIdx.x == 0) part[blockIdx.x] = r;
    }
}

// ---------------------------------------------------------------------------
// 2b. forward with the lines staged in shared memory per timeslice tile
//     (FP32 5-loop energies over spatial planes; fwd_tile_ok).  A block
//     of 128 threads covers FT_TT = 2 time slices x an 8 x 8 patch of the
//     plane (mu, nu) at one value of the third spatial coordinate.  For each
//     shape (a, b) the mu-lines of length a over the patch widened by a
//     below in mu and by b on both sides in nu, and the nu-lines of length b
//     over the patch widened by a on both sides in mu and by b below in nu,
//     are copied into shared memory with cp.async (16 bytes per copy, the
//     next shape's lines in flight while the current shape is computed,
//     double buffered); the four leaves of each site then read their twelve
//     lines from shared memory with 32-bit addresses.
// ---------------------------------------------------------------------------
constexpr int FT_TT = 2, FT_TM = 8, FT_TN = 8, FT_BS = FT_TT * FT_TM * FT_TN;
// matrices of the largest shape's staging area, (3,3): 2 x 11 x 14 x 2
constexpr int FT_MAXPOS = 2 * (FT_TM + 3) * (FT_TN + 6) * FT_TT;
constexpr size_t FT_SMEM = 2 * (size_t)FT_MAXPOS * 5 * sizeof(float4);

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ M3<float> lds_mat(const float4* q) {
    M3<float> m;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float4 v = q[j];
        m.r[2 * j] = v.x;
        m.i[2 * j] = v.y;
        m.r[2 * j + 1] = v.z;
        m.i[2 * j + 1] = v.w;
    }
    const float4 v = q[4];
    m.r[8] = v.x;
    m.i[8] = v.y;
    return m;
}

struct TileGeom {
    int nm, nn, stm, stn, sto;  // extents and site strides along mu, nu; stride of the third direction
};

__global__ void __launch_bounds__(FT_BS, 2)
    k_fwd_tile(Geom g, PlaneArg pa, MatAoS<float> lines, AHAoS<float> kout, double* part) {
    extern __shared__ float4 ft_sm[];
    __shared__ double sh[32];
    const int p = blockIdx.x % pa.np;
    const int mu = sel(pa.mu, p), nu = sel(pa.nu, p), od = 6 - mu - nu;
    TileGeom tg{1, 1, 0, 0, 0};
#pragma unroll
    for (int d = 1; d < 4; ++d) {
        if (d == mu) tg.nm = g.n[d], tg.stm = (int)g.st[d];
        if (d == nu) tg.nn = g.n[d], tg.stn = (int)g.st[d];
        if (d == od) tg.sto = (int)g.st[d];
    }
    int r = blockIdx.x / pa.np;
    const int ntb = g.n[0] / FT_TT, nmb = tg.nm / FT_TM, nnb = tg.nn / FT_TN;
    const int tb = r % ntb;
    r /= ntb;
    const int mb = r % nmb;
    r /= nmb;
    const int nb = r % nnb;
    const int oc = r / nnb;
    const int t0 = tb * FT_TT, m0 = mb * FT_TM, n0 = nb * FT_TN, obase = oc * tg.sto;
    const int tid = threadIdx.x;
    const int tl = tid % FT_TT, ml = (tid / FT_TT) % FT_TM, nl = tid / (FT_TT * FT_TM);
    const int kmu = 3 * sel(pa.slot, mu), knu = 3 * sel(pa.slot, nu);

    // issue the copies of shape k's lines into buf (one commit group)
    auto stage = [&](int k, float4* buf) {
        const int a = c_shapes5[k].a, b = c_shapes5[k].b;
        const int Wm = FT_TN + 2 * b, Rm = (FT_TM + a) * Wm * FT_TT;
        const int Wn = FT_TN + b, Rn = (FT_TM + 2 * a) * Wn * FT_TT;
        // exact quotient by W for the row numbers met here (< 256; W <= 14)
        const unsigned invm = (65536u + Wm - 1) / Wm, invn = (65536u + Wn - 1) / Wn;
        for (int pos = tid; pos < Rm + Rn; pos += FT_BS) {
            const bool isn = pos >= Rm;
            const int q = isn ? pos - Rm : pos;
            const int W = isn ? Wn : Wm;
            const int tt = q % FT_TT, rr = q / FT_TT;
            const int im = (int)(((unsigned)rr * (isn ? invn : invm)) >> 16);
            const int jn = rr - im * W;
            int cm = m0 + im - a;
            cm += cm < 0 ? tg.nm : 0;
            cm -= cm >= tg.nm ? tg.nm : 0;
            int cn = n0 + jn - b;
            cn += cn < 0 ? tg.nn : 0;
            cn -= cn >= tg.nn ? tg.nn : 0;
            const uint32_t site = (uint32_t)(t0 + tt + cm * tg.stm + cn * tg.stn + obase);
            const int plane = isn ? knu + b - 1 : kmu + a - 1;
            const float4* src = lines.unit0_32(site, plane);
            float4* dst = buf + pos * 5;
#pragma unroll
            for (int u = 0; u < 4; ++u) cp_async16(dst + u, src + 32 * u);
            cp_async8(dst + 4, lines.unit4_32(site, plane));
        }
        cp_async_commit();
    };

    M3<float> q = m_zero<float>();
    stage(0, ft_sm);
#pragma unroll 1
    for (int k = 0; k < 7; ++k) {
        const float4* cur = ft_sm + (k & 1) * FT_MAXPOS * 5;
        if (k + 1 < 7) {
            stage(k + 1, ft_sm + ((k + 1) & 1) * FT_MAXPOS * 5);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const int a = c_shapes5[k].a, b = c_shapes5[k].b;
        const int Wm = FT_TN + 2 * b, Rm = (FT_TM + a) * Wm * FT_TT, Wn = FT_TN + b;
        // L(i, j): the line at offset (i mu + j nu) from the thread's site
        auto Lm = [&](int i, int j) { return lds_mat(cur + (((ml + i + a) * Wm + nl + j + b) * FT_TT + tl) * 5); };
        auto Ln = [&](int i, int j) {
            return lds_mat(cur + (Rm + ((ml + i + a) * Wn + nl + j + b) * FT_TT + tl) * 5);
        };
        M3<float> w;
        {
            const M3<float> m00 = Lm(0, 0);
            const M3<float> n00 = Ln(0, 0);
            M3<float> t = mm<false, false>(m00, Ln(a, 0));
            t = mm<false, true>(t, Lm(0, b));
            w = mm<false, true>(t, n00);  // TR
            const M3<float> ma0 = Lm(-a, 0);
            t = mm<false, true>(n00, Lm(-a, b));
            t = mm<false, true>(t, Ln(-a, 0));
            mac<false, false>(w, t, ma0);  // TL
            const M3<float> n0b = Ln(0, -b);
            t = mm<true, true>(ma0, Ln(-a, -b));
            t = mm<false, false>(t, Lm(-a, -b));
            mac<false, false>(w, t, n0b);  // BL
            t = mm<true, false>(n0b, Lm(0, -b));
            t = mm<false, false>(t, Ln(a, -b));
            mac<false, true>(w, t, m00);  // BR
        }
        m_axpy(q, (float)c_shapes5[k].c, w);
        __syncthreads();  // every thread is done with `cur` before it is refilled
    }
    const M3<float> f = ah_quarter(q);
    const double e = -(double)retr_mm<false, false>(f, f);
    const int64_t s = (int64_t)t0 + tl + (int64_t)(m0 + ml) * tg.stm + (int64_t)(n0 + nl) * tg.stn + obase;
    if (kout.p) kout.store(s, p, f);
    if (part) {
        const double rsum = block_sum(e, sh);
        if (threadIdx.x == 0) part[blockIdx.x] = rsum;
    }
}

// The tile kernel is used when the environment sets FLUE_FWD_TILE=1 (read at
// every launch; the L1/L2 kernel is the default, see the measurements beside
// k_fwd) for FP32 5-loop energies over spatial planes whose time extent is
// even and whose plane extents are multiples of the patch.
static bool fwd_tile_ok(const Geom& g, const PlaneArg& pa, int kind, bool fout, bool fits) {
    const char* env = getenv("FLUE_FWD_TILE");
    if (!env || atoi(env) != 1) return false;
    if (kind != 1 || fout || !fits || g.n[0] % FT_TT) return false;
    for (int q = 0; q < pa.np; ++q) {
        const int mu = pa.mu[q], nu = pa.nu[q];
        if (mu == 0 || nu == 0 || g.n[mu] % FT_TM || g.n[nu] % FT_TN) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// 3. line cotangents: one thread per (site, slot, length)
// ---------------------------------------------------------------------------
constexpr int COT_BS = FLUE_COT_BS;



// Cotangent of the line l = L^len_e(P), P the thread's site, Q = P + len e.
// In a plane (e, f) the line is a side of the rectangles of shapes with a
// side len along e and w along f that lie on either side of it (SG = +1:
// towards +f, -1: towards -f).  Every such side, whatever its role (S1, S2,
// S3 = L^+, S4 = L^+), contributes the same form: going on from Q around the
// rectangle, A = the f-line Q -> R1 = Q + SG w f, B = the e-line R1 -> R2 =
// P + SG w f (against e, so daggered), C = the f-line R2 -> P, and
//     dLambda = SG o coef [K(Q) A B C + A K(R1) B C + A B K(R2) C + A B C K(P)]
// with o = +1 when e is the plane's first direction mu, -1 when it is nu
// (the clockwise walks are the daggers of the counter-clockwise leaf words:
// K^+ = -K).  K(Q) and K(P) are the same for every rectangle of the plane,
// so their two terms are summed over the plane's rectangles first:
//     Lambda_plane = K(Q) X + X K(P) + sum_sides SG o coef A Y,
//     X = sum_sides SG o coef A B C,   Y = K(R1) (B C) + B (K(R2) C),
// 4 full products and 2 with an anti-Hermitian K per side, and 2 of the
// latter per plane.  A is the stored line at Q (SG = +1) or the dagger of
// the one at R1 (-1); C the dagger of the one at P (+1) or the one at R2
// (-1); B the dagger of the e-line at R2.  SG is a template argument, so
// every dagger is folded into the products at compile time and only plain
// lines are stored.
template <int SG, typename T, typename I>
__device__ __forceinline__ void line_side(M3<T>& acc, M3<T>& X, T coef, const MatAoS<T>& lines, const AHAoS<T>& kin,
                                          int p, I s, I Q, I off, int pf, int pB) {
    constexpr bool DA = SG < 0, DC = SG > 0;
    const I R1 = Q + off, R2 = s + off;
    T kv[9];
    const M3<T> C = ldm(lines, DC ? s : R2, pf);
    M3<T> t = m_zero<T>();
    ldk(kin, R2, p, kv);
    mac_kx<DC>(t, kv, C);
    const M3<T> B = ldm(lines, R2, pB);
    M3<T> y = mm<true, false>(B, t);
    const M3<T> bc = mm<true, DC>(B, C);
    ldk(kin, R1, p, kv);
    mac_kx(y, kv, bc);
    const M3<T> A = ldm(lines, DA ? R1 : Q, pf);
    const M3<T> abc = mm<DA, false>(A, bc);
    const M3<T> ay = mm<DA, false>(A, y);
    const T sc = SG > 0 ? coef : -coef;
    m_axpy(X, sc, abc);
    m_axpy(acc, sc, ay);
}

template <typename T, typename I>
__global__ void __launch_bounds__(COT_BS, MinBlocks<T>::cot)
    k_linecot(Geom g, PlaneArg pa, MatAoS<T> lines, AHAoS<T> kin, MatAoS<T> lam) {
    // the 3 * nd (direction, length) tasks of one site block run in adjacent
    // blocks, so the neighbourhood they all read stays in L2
    const int ntask = 3 * pa.nd;
    const int task = blockIdx.x % ntask;
    const int64_t s64 = site_block(blockIdx.x / ntask, g, blockDim.x) * blockDim.x + threadIdx.x;
    if (s64 >= g.V) return;
    const I s = (I)s64;
    const int slot = task / 3;
    const int len = task % 3 + 1;
    const int e = sel(pa.dir, slot);
    int c[4];
    site_coords(g, s64, c);
    int ce = 0, ne = 1;
    int64_t ste = 1;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k == e) ce = c[k], ne = g.n[k], ste = g.st[k];
    const I Q = s + (I)((int64_t)wrapd(ce, len, ne) * ste);
    const int pB = 3 * slot + len - 1;
    const int nw = len == 1 ? 3 : 2;
    M3<T> acc = m_zero<T>();
    for (int p = 0; p < pa.np; ++p) {
        const int pmu = sel(pa.mu, p), pnu = sel(pa.nu, p);
        if (pmu != e && pnu != e) continue;
        const int f = pmu == e ? pnu : pmu;
        const T o = pmu == e ? T(1) : T(-1);
        int cf = 0, nf = 1;
        int64_t stf = 1;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k == f) cf = c[k], nf = g.n[k], stf = g.st[k];
        const int kf = 3 * sel(pa.slot, f);
        M3<T> X = m_zero<T>();
#pragma unroll 1
        for (int j = 0; j < nw; ++j) {
            const int w = c_lw_w[len - 1][j];
            const T coef = lw_coef<T>(len, j) * o;
            const int pf = kf + w - 1;
            line_side<+1>(acc, X, coef, lines, kin, p, s, Q, (I)((int64_t)wrapd(cf, w, nf) * stf), pf, pB);
            line_side<-1>(acc, X, coef, lines, kin, p, s, Q, (I)((int64_t)wrapd(cf, -w, nf) * stf), pf, pB);
        }
        T kv[9];
        ldk(kin, Q, p, kv);
        mac_kx(acc, kv, X);
        ldk(kin, s, p, kv);
        mac_xk(acc, X, kv);
    }
    lam.store(s64, 3 * slot + len - 1, acc);
}

// ---------------------------------------------------------------------------
// 4. link cotangents and gradient output: one thread per (site, direction),
//    grid-strided so that a capped grid can write the gradient to host memory
//    beside other kernels
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_linkcot(Geom g, PlaneArg pa, MatAoS<T> lines, MatAoS<T> lam, T scale, int form, RefOut<T> out,
                          bool skip_zero) {
    const int d = blockIdx.y;
    const int slot = sel(pa.slot, d);
    if (slot < 0 && skip_zero) return;
    for (int64_t z = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; z < g.V; z += (int64_t)gridDim.x * blockDim.x) {
        if (slot < 0) {
            out.store(z, d, m_zero<T>());
            continue;
        }
        int c[4];
        site_coords(g, z, c);
        int cd = 0, nd = 1;
        int64_t sd = 1;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k == d) cd = c[k], nd = g.n[k], sd = g.st[k];
        const int64_t zp = z + (int64_t)wrapd(cd, 1, nd) * sd, zm = z + (int64_t)wrapd(cd, -1, nd) * sd,
                      zmm = z + (int64_t)wrapd(cd, -2, nd) * sd;
        const int l1 = 3 * slot, l2 = 3 * slot + 1;
        const M3<T> up = lines.load(zp, l1);
        const M3<T> um = lines.load(zm, l1);
        M3<T> n = lam.load(z, 3 * slot);
        mac<false, false>(n, up, lam.load(z, 3 * slot + 1));
        mac<false, false>(n, lam.load(zm, 3 * slot + 1), um);
        mac<false, false>(n, lines.load(zp, l2), lam.load(z, 3 * slot + 2));
        {
            const M3<T> t = mul(up, lam.load(zm, 3 * slot + 2));
            mac<false, false>(n, t, um);
        }
        mac<false, false>(n, lam.load(zmm, 3 * slot + 2), lines.load(zmm, l2));
        if (form == 0) {
            const M3<T> un = mul(lines.load(z, l1), n);
            out.store(z, d, ta_scaled(un, T(-0.5) * scale));
        } else {
            out.store(z, d, m_scale(dag(n), scale));
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static PlaneArg make_planes(const PlaneSet& ps) {
    PlaneArg pa;
    pa.np = ps.np;
    for (int k = 0; k < 4; ++k) pa.slot[k] = -1, pa.dir[k] = -1;
    pa.nd = 0;
    for (int p = 0; p < ps.np; ++p) {
        pa.mu[p] = ps.mu[p];
        pa.nu[p] = ps.nu[p];
        for (int d : {ps.mu[p], ps.nu[p]})
            if (pa.slot[d] < 0) {
                pa.slot[d] = pa.nd;
                pa.dir[pa.nd] = d;
                pa.nd++;
            }
    }
    return pa;
}

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct EnergyWs {
    size_t lines, kbuf, lam, part, total;
};

static EnergyWs energy_layout(const Geom& g, int prec, const PlaneArg& pa, bool with_force) {
    const bool d = prec == PREC_C128;  // FP64 intermediates
    auto mat = [&](int64_t nk) { return d ? MatAoS<double>::bytes(g.V, nk) : MatAoS<float>::bytes(g.V, nk); };
    auto ah = [&](int64_t nk) { return d ? AHAoS<double>::bytes(g.V, nk) : AHAoS<float>::bytes(g.V, nk); };
    EnergyWs w;
    const int nbx = (int)((g.V + FWD_BS - 1) / FWD_BS);
    w.lines = 0;
    // daggered line copies only when the line cotangents run
    w.kbuf = align256(w.lines + mat(3 * pa.nd));
    w.lam = align256(w.kbuf + (with_force ? ah(pa.np) : 0));
    w.part = align256(w.lam + (with_force ? mat(3 * pa.nd) : 0));
    w.total = align256(w.part + (size_t)pa.np * nbx * sizeof(double));
    return w;
}

size_t energy_ws_bytes(const Geom& g, int prec, const PlaneSet& ps, bool with_force) {
    return energy_layout(g, prec, make_planes(ps), with_force).total;
}

// Optional per-stage timing of the energy pipeline (CUDA events recorded on
// the caller's stream between the stage launches): stage 0 lines, 1 forward
// (+ sum), 2 line cotangents, 3 link cotangents.
static bool g_stage_on = false;
static cudaEvent_t g_stage_ev[5] = {};
static int g_stage_n = 0;

cudaError_t stage_timing_enable(int on) {
    if (on && !g_stage_ev[0]) {
        for (auto& e : g_stage_ev) {
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) return r;
        }
    }
    g_stage_on = on != 0;
    g_stage_n = 0;
    return cudaSuccess;
}

cudaError_t stage_times(double* ms, int maxn, int* n) {
    *n = 0;
    if (!g_stage_on || g_stage_n < 2) return cudaSuccess;
    cudaError_t r = cudaEventSynchronize(g_stage_ev[g_stage_n - 1]);
    if (r != cudaSuccess) return r;
    for (int k = 0; k + 1 < g_stage_n && k < maxn; ++k) {
        float t = 0.f;
        r = cudaEventElapsedTime(&t, g_stage_ev[k], g_stage_ev[k + 1]);
        if (r != cudaSuccess) return r;
        ms[k] = t;
        *n = k + 1;
    }
    return cudaSuccess;
}

static inline void stage_mark(int k, cudaStream_t st) {
    if (g_stage_on) {
        cudaEventRecord(g_stage_ev[k], st);
        g_stage_n = k + 1;
    }
}

// Part 1 of the pipeline: lines, forward (+ energy sum normalised by vnorm),
// line cotangents when `with_force`.
template <class L, typename T>
static cudaError_t energy_fwd_part(const L& U, const Geom& g, const Geom& gs, int t0, const PlaneArg& pa, int kind,
                                   double* out_E, bool with_force, double vnorm, char* ws, const EnergyWs& w,
                                   RefOut<T> fout, cudaStream_t st) {
    MatAoS<T> lines{reinterpret_cast<decltype(MatAoS<T>::p)>(ws + w.lines), g.V};
    AHAoS<T> kb{with_force ? reinterpret_cast<decltype(AHAoS<T>::p)>(ws + w.kbuf) : nullptr, g.V};
    MatAoS<T> lam{reinterpret_cast<decltype(MatAoS<T>::p)>(ws + w.lam), g.V};
    double* part = out_E ? (double*)(ws + w.part) : nullptr;
    const unsigned nbx = (unsigned)((g.V + FWD_BS - 1) / FWD_BS);
    stage_mark(0, st);
    note_launch(), k_lines<L, T><<<dim3((unsigned)((g.V + 127) / 128), pa.nd), 128, 0, st>>>(U, g, gs, t0, pa, lines);
    stage_mark(1, st);
    const PatchArg pt = FLUE_FWD_PATCH ? make_patch(g, pa, FWD_BS) : PatchArg{};
    const bool fits = MatAoS<T>::fits32(g.V, 3 * pa.nd);
    bool tiled = false;
    if constexpr (sizeof(T) == 4) {
        if (fwd_tile_ok(g, pa, kind, fout.p != nullptr, fits)) {
            static_assert(FT_BS == FWD_BS, "the tile forward writes one partial per FWD_BS sites");
            // (the attribute is per function and per device; setting it again is harmless)
            cudaError_t ae = cudaFuncSetAttribute(k_fwd_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FT_SMEM);
            if (ae != cudaSuccess) return ae;
            note_launch(), k_fwd_tile<<<nbx * pa.np, FT_BS, FT_SMEM, st>>>(g, pa, lines, kb, part);
            tiled = true;
        }
    }
    if (!tiled) {
        if (fits)
            note_launch(), k_fwd<T, uint32_t><<<nbx * pa.np, FWD_BS, 0, st>>>(g, pa, kind, pt, lines, kb, fout, part);
        else
            note_launch(), k_fwd<T, int64_t><<<nbx * pa.np, FWD_BS, 0, st>>>(g, pa, kind, pt, lines, kb, fout, part);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (out_E) {
        e = launch_finish_sums(part, (int)(nbx * pa.np), 1, out_E, st, 1.0 / vnorm);
        if (e != cudaSuccess) return e;
    }
    stage_mark(2, st);
    if (!with_force) return cudaSuccess;
    const unsigned nbc = (unsigned)((g.V + COT_BS - 1) / COT_BS);
    if (MatAoS<T>::fits32(g.V, 3 * pa.nd) && AHAoS<T>::fits32(g.V, pa.np))
        note_launch(), k_linecot<T, uint32_t><<<nbc * 3 * pa.nd, COT_BS, 0, st>>>(g, pa, lines, kb, lam);
    else
        note_launch(), k_linecot<T, int64_t><<<nbc * 3 * pa.nd, COT_BS, 0, st>>>(g, pa, lines, kb, lam);
    stage_mark(3, st);
    return cudaGetLastError();
}

// Part 2: link cotangents, gradient of E/vnorm written through `fo`.
template <typename T>
static cudaError_t energy_out_part(const Geom& g, const PlaneArg& pa, double vnorm, int form, char* ws,
                                   const EnergyWs& w, RefOut<T> fo, unsigned max_blocks, cudaStream_t st,
                                   bool skip_zero = false) {
    MatAoS<T> lines{reinterpret_cast<decltype(MatAoS<T>::p)>(ws + w.lines), g.V};
    MatAoS<T> lam{reinterpret_cast<decltype(MatAoS<T>::p)>(ws + w.lam), g.V};
    const T scale = (T)(-1.0 / (2.0 * vnorm));
    unsigned nb = (unsigned)((g.V + 127) / 128);
    if (max_blocks && nb > max_blocks) nb = max_blocks;
    note_launch(), k_linkcot<T><<<dim3(nb, 4), 128, 0, st>>>(g, pa, lines, lam, scale, form, fo, skip_zero);
    stage_mark(4, st);
    return cudaGetLastError();
}

template <class L, typename T>
static cudaError_t energy_impl(const L& U, const Geom& g, const PlaneArg& pa, int kind, double* out_E, void* force,
                               int form, char* ws, const EnergyWs& w, RefOut<T> fout, cudaStream_t st) {
    using C2 = typename V2<T>::type;
    cudaError_t e =
        energy_fwd_part<L, T>(U, g, g, 0, pa, kind, out_E, force != nullptr, (double)g.V, ws, w, fout, st);
    if (e != cudaSuccess || !force) return e;
    RefOut<T> fo{(C2*)force, g.V, 4};
    return energy_out_part<T>(g, pa, (double)g.V, form, ws, w, fo, 0, st);
}

cudaError_t launch_energy(const FieldRef& U, const PlaneSet& ps, double* out_E, void* force, int force_form, void* ws,
                          size_t ws_bytes, cudaStream_t st) {
    const PlaneArg pa = make_planes(ps);
    const EnergyWs w = energy_layout(U.g, U.prec, pa, force != nullptr);
    if (ws_bytes < w.total) return cudaErrorInvalidValue;
    FLUE_DISPATCH_LINKS(U, {
        RefOut<T> none{nullptr, U.g.V, 1};
        return energy_impl<decltype(L), T>(L, U.g, pa, 1, out_E, force, force_form, (char*)ws, w, none, st);
    });
    return cudaSuccess;
}

static bool has_time_plane(const PlaneSet& ps) {
    for (int p = 0; p < ps.np; ++p)
        if (ps.mu[p] == 0 || ps.nu[p] == 0) return true;
    return false;
}

cudaError_t launch_energy_slab_fwd(const FieldRef& U, int t0, int nts, const PlaneSet& ps, int64_t vfull,
                                   double* out_E, bool with_force, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (has_time_plane(ps) || t0 < 0 || nts < 1 || t0 + nts > U.g.n[0]) return cudaErrorInvalidValue;
    const Geom g = make_geom(nts, U.g.n[1], U.g.n[2], U.g.n[3]);
    if (vfull < g.V) return cudaErrorInvalidValue;
    const PlaneArg pa = make_planes(ps);
    const EnergyWs w = energy_layout(g, U.prec, pa, with_force);
    if (ws_bytes < w.total) return cudaErrorInvalidValue;
    FLUE_DISPATCH_LINKS(U, {
        RefOut<T> none{nullptr, g.V, 1};
        return energy_fwd_part<decltype(L), T>(L, g, U.g, t0, pa, 1, out_E, with_force, (double)vfull, (char*)ws, w,
                                               none, st);
    });
    return cudaSuccess;
}

cudaError_t launch_energy_slab_out(const FieldRef& U, const PlaneSet& ps, int64_t vfull, int ntf, int t0, void* force,
                                   int force_form, void* ws, size_t ws_bytes, unsigned max_blocks, cudaStream_t st,
                                   int out_dtype, bool skip_zero) {
    if (has_time_plane(ps) || vfull < U.g.V || t0 < 0 || t0 + U.g.n[0] > ntf) return cudaErrorInvalidValue;
    const PlaneArg pa = make_planes(ps);
    const EnergyWs w = energy_layout(U.g, U.prec, pa, true);
    if (ws_bytes < w.total) return cudaErrorInvalidValue;
    // the gradient array: time extent ntf, the slab's spatial extents (the
    // whole lattice's gradient, or a chunk of ntf time slices of it); vfull
    // only normalises
    const int64_t vout = (int64_t)ntf * (U.g.V / U.g.n[0]);
    if (U.prec == PREC_C128) {
        if (out_dtype != PREC_C128) return cudaErrorInvalidValue;
        RefOut<double> fo{(double2*)force, vout, 4, U.g.n[0], ntf, t0};
        return energy_out_part<double>(U.g, pa, (double)vfull, force_form, (char*)ws, w, fo, max_blocks, st,
                                       skip_zero);
    }
    RefOut<float> fo{(float2*)force, vout, 4, U.g.n[0], ntf, t0};
    if (out_dtype == PREC_C128) fo.p = nullptr, fo.pd = (double2*)force;
    return energy_out_part<float>(U.g, pa, (double)vfull, force_form, (char*)ws, w, fo, max_blocks, st, skip_zero);
}

// ---------------------------------------------------------------------------
// Energy (and gradient) of a device field over time slabs on several streams.
// Plane sets without the time direction (B^2) leave time slices independent,
// so the field is processed as nslab slabs of consecutive time slices, slab
// k on stream k % nstream (the caller's stream and nstream - 1 library
// streams, forked from and joined back to the caller's stream by events).
// The memory-bound stages (lines, link cotangents) of one slab then overlap
// the compute-bound ones of another, and each slab's intermediates are 1/nslab
// of the lattice's.  Per-slab energies are added in slab order by one
// finisher; the gradient is written in place through the slab mapping, so
// both are bitwise independent of the stream schedule.
// ---------------------------------------------------------------------------
namespace {
constexpr int kMaxSlabStreams = 4;
struct SlabStreams {
    std::mutex m;
    cudaStream_t s[kMaxSlabStreams - 1] = {};
    cudaEvent_t fork = nullptr, join[kMaxSlabStreams - 1] = {};
};
std::mutex g_slab_mtx;
SlabStreams* g_slab[64] = {};

cudaError_t slab_streams(SlabStreams** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_slab_mtx);
    if (!g_slab[dev]) {
        SlabStreams* ss = new SlabStreams();
        for (int i = 0; i < kMaxSlabStreams - 1 && e == cudaSuccess; ++i) {
            e = cudaStreamCreateWithFlags(&ss->s[i], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ss->join[i], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ss->fork, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;  // (a failed setup keeps its handles; it is retried on the next call)
        g_slab[dev] = ss;
    }
    *out = g_slab[dev];
    return cudaSuccess;
}

struct SlabWs {
    size_t slot, spart, total;
};
SlabWs slab_ws_layout(const Geom& g, int prec, const PlaneArg& pa, bool with_force, int nslab, int nstream) {
    const int nts = (g.n[0] + nslab - 1) / nslab;
    const Geom gs = make_geom(nts, g.n[1], g.n[2], g.n[3]);
    SlabWs w;
    w.slot = energy_layout(gs, prec, pa, with_force).total;
    w.spart = (size_t)nstream * w.slot;
    w.total = align256(w.spart + (size_t)nslab * sizeof(double));
    return w;
}
}  // namespace

bool stage_timing_on() { return g_stage_on; }

size_t energy_slabs_ws_bytes(const Geom& g, int prec, const PlaneSet& ps, bool with_force, int nslab, int nstream) {
    return slab_ws_layout(g, prec, make_planes(ps), with_force, nslab, nstream).total;
}

cudaError_t launch_energy_slabs(const FieldRef& U, const PlaneSet& ps, double* out_E, void* force, int form, void* ws,
                                size_t ws_bytes, int nslab, int nstream, cudaStream_t st) {
    if (has_time_plane(ps) || nslab < 1 || nslab > U.g.n[0] || nstream < 1 || nstream > kMaxSlabStreams)
        return cudaErrorInvalidValue;
    const PlaneArg pa = make_planes(ps);
    const bool with_force = force != nullptr;
    const SlabWs w = slab_ws_layout(U.g, U.prec, pa, with_force, nslab, nstream);
    if (ws_bytes < w.total) return cudaErrorInvalidValue;
    const int nts = (U.g.n[0] + nslab - 1) / nslab;
    nslab = (U.g.n[0] + nts - 1) / nts;
    if (nstream > nslab) nstream = nslab;
    SlabStreams* ss = nullptr;
    cudaError_t e = slab_streams(&ss);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(ss->m);
    double* spart = out_E ? (double*)((char*)ws + w.spart) : nullptr;
    if ((e = cudaEventRecord(ss->fork, st)) != cudaSuccess) return e;
    for (int i = 1; i < nstream; ++i)
        if ((e = cudaStreamWaitEvent(ss->s[i - 1], ss->fork, 0)) != cudaSuccess) return e;
    for (int k = 0; k < nslab && e == cudaSuccess; ++k) {
        const int i = k % nstream, t0 = k * nts, n = U.g.n[0] - t0 < nts ? U.g.n[0] - t0 : nts;
        cudaStream_t sk = i == 0 ? st : ss->s[i - 1];
        char* slot = (char*)ws + (size_t)i * w.slot;
        e = launch_energy_slab_fwd(U, t0, n, ps, U.g.V, spart ? spart + k : nullptr, with_force, slot, w.slot, sk);
        if (e == cudaSuccess && with_force) {
            const FieldRef Us{U.links, make_geom(n, U.g.n[1], U.g.n[2], U.g.n[3]), U.prec};
            e = launch_energy_slab_out(Us, ps, U.g.V, U.g.n[0], t0, force, form, slot, w.slot, 0, sk,
                                       U.prec == PREC_C128 ? PREC_C128 : PREC_C64);
        }
    }
    // join every library stream back into the caller's stream, also on error
    for (int i = 1; i < nstream; ++i) {
        cudaError_t r = cudaEventRecord(ss->join[i - 1], ss->s[i - 1]);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(st, ss->join[i - 1], 0);
        if (e == cudaSuccess) e = r;
    }
    if (e == cudaSuccess && out_E) e = launch_finish_sums(spart, nslab, 1, out_E, st, 1.0);
    return e;
}

// F_munu of one plane: kind 0 = clover (cloverLoopMuNuCoord), 1 = 5-loop
// (Loop5MuNuCoord).  Output (NT,NX,NY,NZ,3,3) in the field's compute dtype.
cudaError_t launch_fmunu(const FieldRef& U, int kind, int mu, int nu, void* out, void* ws, size_t ws_bytes,
                         cudaStream_t st) {
    PlaneSet ps;
    ps.np = 1;
    ps.mu[0] = mu;
    ps.nu[0] = nu;
    const PlaneArg pa = make_planes(ps);
    const EnergyWs w = energy_layout(U.g, U.prec, pa, false);
    if (ws_bytes < w.total) return cudaErrorInvalidValue;
    FLUE_DISPATCH_LINKS(U, {
        using C2 = typename V2<T>::type;
        RefOut<T> fo{(C2*)out, U.g.V, 1};
        return energy_impl<decltype(L), T>(L, U.g, pa, kind, nullptr, nullptr, 0, (char*)ws, w, fo, st);
    });
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Wilson plaquette action S = sum_{x,mu<nu} Re Tr P_munu(x) and its gradient:
// N_mu(x) = sum_{nu != mu} [U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+
//                           + U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu)]
// ---------------------------------------------------------------------------
constexpr int PF_BS = 128;
int plaqforce_blocks(const Geom& g) { return (int)((g.V + PF_BS - 1) / PF_BS); }

// Staple sum and gradient of direction MU at site s; MU and the staple
// directions are compile-time, so every coordinate and stride is a register.
template <int MU, class L, typename T>
__device__ __forceinline__ double plaqforce_dir(const L& U, const Geom& g, int64_t s, const int c[4], int form,
                                                const RefOut<T>& out) {
    const int64_t sp = s + (int64_t)wrapd(c[MU], 1, g.n[MU]) * g.st[MU];
    const M3<T> u = U.load(s, MU);
    M3<T> n = m_zero<T>();
    double acc = 0.0;
#pragma unroll
    for (int nu = 0; nu < 4; ++nu) {
        if (nu == MU) continue;
        const int64_t dn1 = (int64_t)wrapd(c[nu], 1, g.n[nu]) * g.st[nu];
        const int64_t dm1 = (int64_t)wrapd(c[nu], -1, g.n[nu]) * g.st[nu];
        const M3<T> up = mm<false, true>(U.load(sp, nu), U.load(s + dn1, MU));
        const M3<T> upper = mm<false, true>(up, U.load(s, nu));
        if (nu > MU) acc += (double)retr_mm<false, false>(u, upper);
        m_add(n, upper);
        const M3<T> dn = mm<true, true>(U.load(sp + dm1, nu), U.load(s + dm1, MU));
        mac<false, false>(n, dn, U.load(s + dm1, nu));
    }
    if (out.p) {
        if (form == 0)
            out.store(s, MU, ta_scaled(mul(u, n), T(-0.5)));
        else
            out.store(s, MU, dag(n));
    }
    return acc;
}

// Minimum resident blocks per SM (register cap) of k_plaqforce, measured on
// GB300 at 32^3x64: c64 2.03 ms per call with runtime directions (80-byte
// local frame), 1.64 with compile-time ones, 1.48 capped at 3 blocks; r12
// 1.27 -> 1.15 capped at 4; FP64 keeps its registers (21.1 ms either way).
template <class L, typename T>
struct PfMinBlocks {
    static constexpr int v = sizeof(T) == 4 ? 3 : 1;
};
template <>
struct PfMinBlocks<R12Links, float> {
    static constexpr int v = 4;
};

template <class L, typename T>
__global__ void __launch_bounds__(PF_BS, PfMinBlocks<L, T>::v)
    k_plaqforce(L U, Geom g, int form, RefOut<T> out, double* part) {
    __shared__ double sh[32];
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (s < g.V) {
        int c[4];
        site_coords(g, s, c);
        switch (blockIdx.y) {
            case 0: acc = plaqforce_dir<0>(U, g, s, c, form, out); break;
            case 1: acc = plaqforce_dir<1>(U, g, s, c, form, out); break;
            case 2: acc = plaqforce_dir<2>(U, g, s, c, form, out); break;
            default: acc = plaqforce_dir<3>(U, g, s, c, form, out); break;
        }
    }
    if (part) {
        const double r = block_sum(acc, sh);
        if (threadIdx.x == 0) part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = r;
    }
}

cudaError_t launch_plaquette_force(const FieldRef& U, double* part, double* out_S, void* force, int force_form,
                                   cudaStream_t st) {
    const int nb = plaqforce_blocks(U.g);
    FLUE_DISPATCH_LINKS(U, {
        using C2 = typename V2<T>::type;
        RefOut<T> fo{(C2*)force, U.g.V, 4};
        note_launch(), k_plaqforce<decltype(L), T><<<dim3(nb, 4), PF_BS, 0, st>>>(L, U.g, force_form, fo, out_S ? part : nullptr);
    });
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !out_S) return e;
    return launch_finish_sums(part, 4 * nb, 1, out_S, st);
}

FLUE_OOB_READER(force)

}  // namespace flue
