// observables.cu -- layout conversion, SU(3) batch products, and the scalar
// observables of src/wloops.F90: plaquette (:915-1017, same observable as
// genPlaquette :59-127), polyakov (:1019-1069), wmunu / wmunutau
// (:567-791), genericPath (:20-57) and the Landau-gauge mean link used by
// uzerobar.  Every scalar is accumulated per thread in FP64 (the FP32 path
// computes link products in FP32 and converts each per-site trace), reduced
// per block with warp shuffles, and finished by a one-block kernel that adds
// the block partials in index order, so results are bitwise reproducible for
// a given lattice size.
#include <atomic>

#include "flue_internal.h"

namespace flue {

static inline int grid_for(int64_t n, int bs, int cap) {
    int64_t b = (n + bs - 1) / bs;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

int device_sms() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 152;
    }
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
        cudaGetLastError();
        return 152;
    }
    cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

// Grid-strided reductions run 4 blocks per SM of the current device, at most
// kMaxRedBlocks; their partial-sum workspaces are sized for kMaxRedBlocks.
static int red_cap() {
    const int c = 4 * device_sms();
    return c > kMaxRedBlocks ? kMaxRedBlocks : c;
}

// ---------------------------------------------------------------------------
// reduction finisher
// ---------------------------------------------------------------------------
__global__ void k_finish_sums(const double* __restrict__ part, int nparts, double scale, double* __restrict__ out) {
    __shared__ double sh[32];
    const double* p = part + (int64_t)blockIdx.x * nparts;
    double acc = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += p[i];
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = scale == 1.0 ? r : r * scale;
}

cudaError_t launch_finish_sums(const double* partial, int nparts, int nout, double* out, cudaStream_t st, double scale) {
    note_launch(), k_finish_sums<<<nout, 256, 0, st>>>(partial, nparts, scale, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// pack: arbitrary-strided (t,x,y,z,mu,a,b) complex128/complex64 -> device
// layout, optionally reunitarised.  One thread per (site, mu), grid-strided
// so that a capped grid can stream a field in beside other kernels.
// ---------------------------------------------------------------------------
struct Strides7 {
    int64_t s[7];
};

template <typename SRC>
__device__ __forceinline__ void pack_one(const SRC* __restrict__ src, const Strides7& sd, const Geom& g,
                                         void* __restrict__ dst, int dst_prec, int reun, int64_t idx) {
    const int64_t s = idx % g.V;
    const int mu = (int)(idx / g.V);
    int c[4];
    site_coords(g, s, c);
    const int64_t base = c[0] * sd.s[0] + c[1] * sd.s[1] + c[2] * sd.s[2] + c[3] * sd.s[3] + mu * sd.s[4];
    double r[3][3], im[3][3];
    // reconstruct-12 keeps the first two rows: without reunitarisation the
    // third row is not read at all (in the reference's layout its elements
    // are planes of their own, a third of the field's bytes -- a host field
    // read over NVLink-C2C moves 2/3 of its size)
    const int na = (dst_prec == PREC_R12 && !reun) ? 2 : 3;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            r[a][b] = im[a][b] = 0.0;
            if (a < na) {
                const SRC v = src[base + a * sd.s[5] + b * sd.s[6]];
                r[a][b] = (double)v.x;
                im[a][b] = (double)v.y;
            }
        }
    if (reun) fix_su3_rows(r, im);
    if (dst_prec == PREC_C128) {
        double2* o = (double2*)dst + s + g.V * mu;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) o[4 * g.V * (a + 3 * b)] = make_double2(r[a][b], im[a][b]);
    } else if (dst_prec == PREC_C64) {
        float2* o = (float2*)dst + s + g.V * mu;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) o[4 * g.V * (a + 3 * b)] = make_float2((float)r[a][b], (float)im[a][b]);
    } else {
        float4* o = (float4*)dst + s + g.V * (3 * mu);
        o[0] = make_float4((float)r[0][0], (float)im[0][0], (float)r[0][1], (float)im[0][1]);
        o[g.V] = make_float4((float)r[0][2], (float)im[0][2], (float)r[1][0], (float)im[1][0]);
        o[2 * g.V] = make_float4((float)r[1][1], (float)im[1][1], (float)r[1][2], (float)im[1][2]);
    }
}

template <typename SRC>
__global__ void k_pack(const SRC* __restrict__ src, Strides7 sd, Geom g, void* __restrict__ dst, int dst_prec, int reun,
                       int mu0) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (4 - mu0) * g.V;
         idx += (int64_t)gridDim.x * blockDim.x)
        pack_one(src, sd, g, dst, dst_prec, reun, idx + mu0 * g.V);
}

cudaError_t launch_pack(const void* src, int src_dtype, const int64_t strides[7], const Geom& g, void* dst, int dst_prec,
                        int reunitarise, cudaStream_t st, unsigned max_blocks, int mu0) {
    Strides7 sd;
    for (int k = 0; k < 7; ++k) sd.s[k] = strides[k];
    if (mu0 < 0 || mu0 > 3) return cudaErrorInvalidValue;
    const int64_t n = (4 - mu0) * g.V;
    const int bs = 256;
    unsigned nb = (unsigned)((n + bs - 1) / bs);
    if (max_blocks && nb > max_blocks) nb = max_blocks;
    if (src_dtype == PREC_C128)
        note_launch(), k_pack<double2><<<nb, bs, 0, st>>>((const double2*)src, sd, g, dst, dst_prec, reunitarise, mu0);
    else
        note_launch(), k_pack<float2><<<nb, bs, 0, st>>>((const float2*)src, sd, g, dst, dst_prec, reunitarise, mu0);
    return cudaGetLastError();
}

// in-place FixSU3Matrix of a device field (any precision)
__global__ void k_fix_field(void* links, Geom g, int prec) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 4 * g.V) return;
    const int64_t s = idx % g.V;
    const int mu = (int)(idx / g.V);
    double r[3][3], im[3][3];
    if (prec == PREC_C128) {
        double2* o = (double2*)links + s + g.V * mu;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const double2 v = o[4 * g.V * (a + 3 * b)];
                r[a][b] = v.x;
                im[a][b] = v.y;
            }
        fix_su3_rows(r, im);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) o[4 * g.V * (a + 3 * b)] = make_double2(r[a][b], im[a][b]);
    } else if (prec == PREC_C64) {
        float2* o = (float2*)links + s + g.V * mu;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const float2 v = o[4 * g.V * (a + 3 * b)];
                r[a][b] = v.x;
                im[a][b] = v.y;
            }
        fix_su3_rows(r, im);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) o[4 * g.V * (a + 3 * b)] = make_float2((float)r[a][b], (float)im[a][b]);
    } else {
        float4* o = (float4*)links + s + g.V * (3 * mu);
        const float4 q0 = o[0], q1 = o[g.V], q2 = o[2 * g.V];
        r[0][0] = q0.x; im[0][0] = q0.y; r[0][1] = q0.z; im[0][1] = q0.w;
        r[0][2] = q1.x; im[0][2] = q1.y; r[1][0] = q1.z; im[1][0] = q1.w;
        r[1][1] = q2.x; im[1][1] = q2.y; r[1][2] = q2.z; im[1][2] = q2.w;
        fix_su3_rows(r, im);
        o[0] = make_float4((float)r[0][0], (float)im[0][0], (float)r[0][1], (float)im[0][1]);
        o[g.V] = make_float4((float)r[0][2], (float)im[0][2], (float)r[1][0], (float)im[1][0]);
        o[2 * g.V] = make_float4((float)r[1][1], (float)im[1][1], (float)r[1][2], (float)im[1][2]);
    }
}

cudaError_t launch_fix_field(void* links, const Geom& g, int prec, cudaStream_t st) {
    const int64_t n = 4 * g.V;
    note_launch(), k_fix_field<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(links, g, prec);
    return cudaGetLastError();
}

// unpack: device layout -> reference layout (complex128 or complex64)
template <class L, typename T, typename D2>
__global__ void k_unpack(L U, Geom g, D2* __restrict__ dst) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 4 * g.V) return;
    const int64_t s = idx % g.V;
    const int mu = (int)(idx / g.V);
    const M3<T> m = U.load(s, mu);
    D2* o = dst + s + g.V * mu;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            D2 v;
            v.x = m.r[3 * a + b];
            v.y = m.i[3 * a + b];
            o[4 * g.V * (a + 3 * b)] = v;
        }
}

cudaError_t launch_unpack(const FieldRef& U, void* dst, int dst_dtype, cudaStream_t st) {
    const int64_t n = 4 * U.g.V;
    const unsigned nb = (unsigned)((n + 255) / 256);
    FLUE_DISPATCH_LINKS(U, {
        if (dst_dtype == PREC_C128)
            note_launch(), k_unpack<decltype(L), T, double2><<<nb, 256, 0, st>>>(L, U.g, (double2*)dst);
        else
            note_launch(), k_unpack<decltype(L), T, float2><<<nb, 256, 0, st>>>(L, U.g, (float2*)dst);
    });
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// batched MultiplyMatMat (src/SU3MatrixOps.f90:19-37) / MultiplyMatdagMatdag
// (:39-58; its code forms conj(sum_k L(k,i) R(j,k)) = (L^+ R^+)(i,j), although
// its comment reads (L R)^+): n matrices of 9 complex, Fortran order (a + 3b).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_matmul_batch(const typename V2<T>::type* __restrict__ l, const typename V2<T>::type* __restrict__ r,
                               typename V2<T>::type* __restrict__ o, int64_t n, int dagger) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    M3<T> A, B;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const auto x = l[9 * j + a + 3 * b];
            const auto y = r[9 * j + a + 3 * b];
            A.r[3 * a + b] = x.x;
            A.i[3 * a + b] = x.y;
            B.r[3 * a + b] = y.x;
            B.i[3 * a + b] = y.y;
        }
    // MultiplyMatdagMatdag computes L^+ R^+ (src/SU3MatrixOps.f90:47-57)
    const M3<T> C = dagger ? mm<true, true>(A, B) : mul(A, B);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            typename V2<T>::type v;
            v.x = C.r[3 * a + b];
            v.y = C.i[3 * a + b];
            o[9 * j + a + 3 * b] = v;
        }
}

cudaError_t launch_matmul_batch(const void* l, const void* r, void* o, int64_t n, int dtype, int dagger, cudaStream_t st) {
    const unsigned nb = (unsigned)((n + 127) / 128);
    if (dtype == PREC_C128)
        note_launch(), k_matmul_batch<double><<<nb, 128, 0, st>>>((const double2*)l, (const double2*)r, (double2*)o, n, dagger);
    else
        note_launch(), k_matmul_batch<float><<<nb, 128, 0, st>>>((const float2*)l, (const float2*)r, (float2*)o, n, dagger);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// plaquette over planes mu in [mu0,mu1], nu in (mu,nu1] (0-based):
// Re Tr[(U_mu(x) U_nu(x+mu)) (U_mu(x+nu) U_nu(x))^+]  (src/wloops.F90:960-1005)
// ---------------------------------------------------------------------------
constexpr int RED_BS = 256;

int plaquette_blocks(const Geom& g) { return grid_for(g.V, RED_BS, red_cap()); }
int plaquette_slots(const Geom& g) { return grid_for(g.V, RED_BS, kMaxRedBlocks); }

// FP32: at most 128 registers (two 256-thread blocks per SM): measured on
// GB300 at 32^3x64, all planes, c64 0.53 -> 0.36 ms per call against the
// unbounded unrolled kernel's 0.45 ms; FP64 keeps its registers (bound by the
// FP64 pipe, it spills under the cap)
#ifndef FLUE_PLAQ_MINB
#define FLUE_PLAQ_MINB 2
#endif
template <class L, typename T>
__global__ void __launch_bounds__(RED_BS, sizeof(T) == 4 ? FLUE_PLAQ_MINB : 1)
    k_plaquette(L U, Geom g, int mu0, int mu1, int nu1, double* __restrict__ part) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.V; s += (int64_t)gridDim.x * blockDim.x) {
        int c[4];
        site_coords(g, s, c);
        int64_t sp[4];  // s + mu for every direction (compile-time indices only)
#pragma unroll
        for (int d = 0; d < 4; ++d) sp[d] = s + disp(g, d, c[d], 1);
        // the six planes unrolled; the requested range selects them at run time
#pragma unroll
        for (int mu = 0; mu < 3; ++mu) {
            if (mu < mu0 || mu > mu1) continue;
            const M3<T> umu = U.load(s, mu);
#pragma unroll
            for (int nu = mu + 1; nu < 4; ++nu) {
                if (nu > nu1) continue;
                // MultiplyMatdagMatdag(Umu_xnu, Unu_x) = Umu_xnu^+ Unu_x^+ = (Unu_x Umu_xnu)^+
                const M3<T> a = mul(umu, U.load(sp[mu], nu));
                const M3<T> b = mul(U.load(s, nu), U.load(sp[nu], mu));
                acc += (double)retr_mm<false, true>(a, b);
            }
        }
    }
    const double r = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

cudaError_t launch_plaquette(const FieldRef& U, int mu0, int mu1, int nu1, double* part, double* out, cudaStream_t st) {
    const int nb = plaquette_blocks(U.g);
    FLUE_DISPATCH_LINKS(U, note_launch(), k_plaquette<decltype(L), T><<<nb, RED_BS, 0, st>>>(L, U.g, mu0, mu1, nu1, part));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_finish_sums(part, nb, 1, out, st);
}

// ---------------------------------------------------------------------------
// Polyakov loop: ordered product of U_t over t = 1..NT at every spatial site
// (src/wloops.F90:1043-1066); out2 = [sum Re Tr, sum Im Tr].
// ---------------------------------------------------------------------------
// FP32: one warp per spatial site: lane l multiplies the links of its time
// range [l k, (l+1) k), k = ceil(NT/32) (the lanes read consecutive links,
// so the loads coalesce), then five shuffle levels multiply neighbouring
// partial products in order, P[0,2w) = P[0,w) P[w,2w); lanes past NT hold
// the identity.  Same ordered product, associated as a tree.  FP64: one
// thread per spatial site walks its column (the tree issues ~3x the FP64
// products per site and the FP64 pipe is the bound: 32^3x64 0.53 ms serial
// against 1.11 ms as a tree; FP32 0.17 -> 0.13 ms per call as a tree).
static int polyakov_blocks_serial(const Geom& g) { return grid_for(g.V / g.n[0], RED_BS, red_cap()); }
int polyakov_blocks(const Geom& g) { return grid_for(g.V / g.n[0], RED_BS / 32, red_cap()); }
int polyakov_slots(const Geom& g) { return grid_for(g.V / g.n[0], RED_BS / 32, kMaxRedBlocks); }  // the larger grid

template <typename T>
__device__ __forceinline__ M3<T> shfl_down_m3(const M3<T>& m, int off) {
    M3<T> o;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        o.r[k] = __shfl_down_sync(0xffffffffu, m.r[k], off);
        o.i[k] = __shfl_down_sync(0xffffffffu, m.i[k], off);
    }
    return o;
}

template <class L, typename T>
__global__ void __launch_bounds__(RED_BS) k_polyakov(L U, Geom g, double* __restrict__ part) {
    __shared__ double sh[32];
    double accr = 0.0, acci = 0.0;
    const int nt = g.n[0];
    const int64_t V3 = g.V / nt;
    const int lane = threadIdx.x & 31;
    const int k = (nt + 31) / 32;
    const int t0 = lane * k, t1 = min(nt, t0 + k);
    if (sizeof(T) == 8) {
        for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < V3; r += (int64_t)gridDim.x * blockDim.x) {
            const int64_t s0 = r * nt;
            M3<T> p = U.load(s0, 0);
            for (int t = 1; t < nt; ++t) p = mul(p, U.load(s0 + t, 0));
            accr += (double)retr(p);
            acci += (double)(p.i[0] + p.i[4] + p.i[8]);
        }
    } else {
        const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
        for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < V3; r += warps) {
            const int64_t s0 = r * nt;
            M3<T> p = m_ident<T>();
            if (t0 < nt) {
                p = U.load(s0 + t0, 0);
                for (int t = t0 + 1; t < t1; ++t) p = mul(p, U.load(s0 + t, 0));
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const M3<T> q = shfl_down_m3(p, off);
                if ((lane & (2 * off - 1)) == 0) p = mul(p, q);
            }
            if (lane == 0) {
                accr += (double)retr(p);
                acci += (double)(p.i[0] + p.i[4] + p.i[8]);
            }
        }
    }
    double a = block_sum(accr, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
    a = block_sum(acci, sh);
    if (threadIdx.x == 0) part[gridDim.x + blockIdx.x] = a;
}

cudaError_t launch_polyakov(const FieldRef& U, double* part, double* out2, cudaStream_t st) {
    const int nb = U.prec == PREC_C128 ? polyakov_blocks_serial(U.g) : polyakov_blocks(U.g);
    FLUE_DISPATCH_LINKS(U, note_launch(), k_polyakov<decltype(L), T><<<nb, RED_BS, 0, st>>>(L, U.g, part));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_finish_sums(part, nb, 2, out2, st);
}

// ---------------------------------------------------------------------------
// nMu x nNu Wilson loop at every site (tau < 0) or on the slice t = tau
// (src/wloops.F90:599-675 and :711-789).
// ---------------------------------------------------------------------------
int wloop_blocks(const Geom& g) { return grid_for(g.V, RED_BS, red_cap()); }
int wloop_slots(const Geom& g) { return grid_for(g.V, RED_BS, kMaxRedBlocks); }

// coordinate, extent and stride of direction d (runtime) without
// runtime-indexed arrays (they would go to local memory)
__device__ __forceinline__ void dir_of(const Geom& g, const int c[4], int d, int& cd, int& nd, int64_t& sd) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k == d) cd = c[k], nd = g.n[k], sd = g.st[k];
}

// product U_d(x) U_d(x+d) ... of n links starting at site s, whose
// coordinate along d is cd (extent nd, stride sd)
template <class L, typename T>
__device__ __forceinline__ M3<T> line_walk(const L& U, int64_t s, int d, int cd, int nd, int64_t sd, int n) {
    M3<T> p = U.load(s, d);
    for (int k = 1; k < n; ++k) {
        s += (cd + 1 == nd) ? -(int64_t)(nd - 1) * sd : sd;
        cd = (cd + 1 == nd) ? 0 : cd + 1;
        p = mul(p, U.load(s, d));
    }
    return p;
}

template <class L, typename T>
__global__ void __launch_bounds__(RED_BS)
    k_wloop(L U, Geom g, int tau, int mu, int nu, int nmu, int nnu, double* __restrict__ part) {
    __shared__ double sh[32];
    double acc = 0.0;
    const int64_t nsites = tau < 0 ? g.V : g.V / g.n[0];
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nsites; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = tau < 0 ? j : (int64_t)tau + j * g.n[0];
        int c[4];
        site_coords(g, s, c);
        int cm = 0, nm = 1, cn = 0, nn = 1;
        int64_t sm = 1, sn = 1;
        dir_of(g, c, mu, cm, nm, sm);
        dir_of(g, c, nu, cn, nn, sn);
        const int cm2 = (int)(((int64_t)cm + nmu) % nm), cn2 = (int)(((int64_t)cn + nnu) % nn);
        const int64_t smu = s + (int64_t)(cm2 - cm) * sm, snu = s + (int64_t)(cn2 - cn) * sn;
        const M3<T> a = line_walk<L, T>(U, s, mu, cm, nm, sm, nmu);
        const M3<T> b = line_walk<L, T>(U, smu, nu, cn, nn, sn, nnu);   // x + nMu mu: same nu coordinate
        const M3<T> cc = line_walk<L, T>(U, snu, mu, cm, nm, sm, nmu);  // x + nNu nu: same mu coordinate
        const M3<T> d = line_walk<L, T>(U, s, nu, cn, nn, sn, nnu);
        // Re Tr[(A B) (C^+ D^+)] with C^+ D^+ = (D C)^+  (MultiplyMatdagMatdag, :669)
        const M3<T> ab = mul(a, b);
        const M3<T> dc = mul(d, cc);
        acc += (double)retr_mm<false, true>(ab, dc);
    }
    const double r = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

cudaError_t launch_wloop(const FieldRef& U, int tau, int mu, int nu, int nmu, int nnu, double* part, double* out,
                         cudaStream_t st) {
    const int nb = wloop_blocks(U.g);
    FLUE_DISPATCH_LINKS(U, note_launch(), k_wloop<decltype(L), T><<<nb, RED_BS, 0, st>>>(L, U.g, tau, mu, nu, nmu, nnu, part));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const double norm = tau < 0 ? (double)U.g.V : (double)(U.g.V / U.g.n[0]);
    return launch_finish_sums(part, nb, 1, out, st, 1.0 / norm);
}

// ---------------------------------------------------------------------------
// W_munu table: wmunu(mu, nu, R, T) for every R <= rmax, T <= tmax at once
// (the reference evaluates src/wloops.F90:679-791 once per (R, T), walking
// every line anew).  k_wt_lines stores per site the mu-lines L_R = U_mu(x)
// ... U_mu(x+(R-1)mu) and the nu-lines L_T, built incrementally; k_wt_loops
// forms each loop from four stored lines, Re Tr[(A B)(D C)^+] with A = L_R(x),
// B = L_T(x+R mu), C = L_R(x+T nu), D = L_T(x) -- the formula of k_wloop --
// with the rmax * tmax tasks of one site block in adjacent blocks (the
// neighbour lines they read stay in L2).
// ---------------------------------------------------------------------------
constexpr int WT_BS = 128;

template <class L, typename T>
__global__ void k_wt_lines(L U, Geom g, int mu, int nu, int rmax, int tmax, MatAoS<T> lines) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.V) return;
    int c[4];
    site_coords(g, s, c);
    for (int pass = 0; pass < 2; ++pass) {
        const int d = pass ? nu : mu, n = pass ? tmax : rmax, k0 = pass ? rmax : 0;
        int cd = 0, nd = 1;
        int64_t sd = 1;
        dir_of(g, c, d, cd, nd, sd);
        int64_t sw = s;
        M3<T> p = U.load(sw, d);
        lines.store(s, k0, p);
        for (int k = 1; k < n; ++k) {
            sw += (cd + 1 == nd) ? -(int64_t)(nd - 1) * sd : sd;
            cd = (cd + 1 == nd) ? 0 : cd + 1;
            p = mul(p, U.load(sw, d));
            lines.store(s, k0 + k, p);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(WT_BS) k_wt_loops(Geom g, int mu, int nu, int rmax, int tmax, MatAoS<T> lines,
                                                    double* __restrict__ part) {
    __shared__ double sh[32];
    const int nrt = rmax * tmax;
    const int rt = blockIdx.x % nrt;
    const int sb = blockIdx.x / nrt;
    const int nsb = gridDim.x / nrt;
    const int R = rt / tmax + 1, Tl = rt % tmax + 1;
    const int64_t s = (int64_t)sb * WT_BS + threadIdx.x;
    double acc = 0.0;
    if (s < g.V) {
        int c[4];
        site_coords(g, s, c);
        int cm = 0, nm = 1, cn = 0, nn = 1;
        int64_t sm = 1, sn = 1;
        dir_of(g, c, mu, cm, nm, sm);
        dir_of(g, c, nu, cn, nn, sn);
        const int64_t sR = s + (int64_t)((cm + R) % nm - cm) * sm;
        const int64_t sT = s + (int64_t)((cn + Tl) % nn - cn) * sn;
        const M3<T> ab = mul(lines.load(s, R - 1), lines.load(sR, rmax + Tl - 1));
        const M3<T> dc = mul(lines.load(s, rmax + Tl - 1), lines.load(sT, R - 1));
        acc = (double)retr_mm<false, true>(ab, dc);
    }
    const double r = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(int64_t)rt * nsb + sb] = r;
}

// the stored mu- and nu-lines of every length, rounded to 256 bytes
static size_t wt_lines_bytes(const Geom& g, int prec, int rmax, int tmax) {
    const size_t b = prec == PREC_C128 ? MatAoS<double>::bytes(g.V, rmax + tmax) : MatAoS<float>::bytes(g.V, rmax + tmax);
    return (b + 255) & ~(size_t)255;
}

size_t wmunu_table_ws_bytes(const Geom& g, int prec, int rmax, int tmax) {
    const size_t nsb = (size_t)((g.V + WT_BS - 1) / WT_BS);
    const size_t lines = wt_lines_bytes(g, prec, rmax, tmax);
    return lines + (((size_t)rmax * tmax * nsb * sizeof(double) + 255) & ~(size_t)255);
}

cudaError_t launch_wmunu_table(const FieldRef& U, int mu, int nu, int rmax, int tmax, double* out, void* ws,
                               cudaStream_t st) {
    const Geom& g = U.g;
    const size_t lines_b = wt_lines_bytes(g, U.prec, rmax, tmax);
    double* part = (double*)((char*)ws + lines_b);
    const unsigned nsb = (unsigned)((g.V + WT_BS - 1) / WT_BS);
    const unsigned nrt = (unsigned)(rmax * tmax);
    FLUE_DISPATCH_LINKS(U, {
        MatAoS<T> ln{reinterpret_cast<decltype(MatAoS<T>::p)>(ws), g.V};
        note_launch(), k_wt_lines<decltype(L), T><<<nsb, WT_BS, 0, st>>>(L, g, mu, nu, rmax, tmax, ln);
        note_launch(), k_wt_loops<T><<<nsb * nrt, WT_BS, 0, st>>>(g, mu, nu, rmax, tmax, ln, part);
    });
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_finish_sums(part, (int)nsb, (int)nrt, out, st, 1.0 / (double)g.V);
}

// ---------------------------------------------------------------------------
// genericPath (src/wloops.F90:20-57) at every site or one site.  Output is the
// TRANSPOSE of the ordered product, in the layout (NT,NX,NY,NZ,3,3) (or one
// 3x3 Fortran-ordered matrix), complex128 for FP64 fields, complex64 else.
// ---------------------------------------------------------------------------
constexpr int MAX_PATH = 256;
struct PathArg {
    int n;
    int step[MAX_PATH];  // +-(mu+1)
};

template <class L, typename T>
__global__ void k_genericpath(L U, Geom g, PathArg path, int64_t s_single, typename V2<T>::type* __restrict__ out) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool single = s_single >= 0;
    if (single ? j > 0 : j >= g.V) return;
    const int64_t s0 = single ? s_single : j;
    int c[4];
    site_coords(g, s0, c);
    int64_t s = s0;
    M3<T> p = m_ident<T>();
    // one periodic step of +-1 along direction mu (runtime); the branch over
    // the four directions keeps coordinates and strides in registers
    auto move = [&](int mu, int dir) {
#pragma unroll
        for (int d = 0; d < 4; ++d)
            if (d == mu) {
                const int n = g.n[d];
                int cd = c[d] + dir;
                int64_t ds = dir * g.st[d];
                if (cd < 0) cd += n, ds += (int64_t)n * g.st[d];
                if (cd >= n) cd -= n, ds -= (int64_t)n * g.st[d];
                c[d] = cd;
                s += ds;
            }
    };
    for (int k = 0; k < path.n; ++k) {
        const int st = path.step[k];
        if (st < 0) {
            const int mu = -st - 1;
            move(mu, -1);
            p = mm<false, true>(p, U.load(s, mu));
        } else {
            const int mu = st - 1;
            p = mul(p, U.load(s, mu));
            move(mu, 1);
        }
    }
    RefOut<T> o{out, single ? 1 : g.V, 1};
    o.store(single ? 0 : s0, 0, transp(p));
}

cudaError_t launch_genericpath(const FieldRef& U, const int* path_host, int npath, const int* coord_host, void* out,
                               cudaStream_t st) {
    PathArg pa;
    pa.n = npath;
    for (int k = 0; k < npath; ++k) pa.step[k] = path_host[k];
    int64_t ss = -1;
    if (coord_host) {
        ss = (int64_t)(coord_host[0] - 1) + U.g.st[1] * (coord_host[1] - 1) + U.g.st[2] * (coord_host[2] - 1) +
             U.g.st[3] * (coord_host[3] - 1);
    }
    const unsigned nb = coord_host ? 1u : (unsigned)((U.g.V + 127) / 128);
    FLUE_DISPATCH_LINKS(U, note_launch(), k_genericpath<decltype(L), T><<<nb, 128, 0, st>>>(L, U.g, pa, ss, (typename V2<T>::type*)out));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Landau-gauge mean link: per direction sum over sites of
// Re Tr(G(x) U_mu(x) G(x+mu)^+), G in (NT,NX,NY,NZ,3,3) layout.
// ---------------------------------------------------------------------------
int meanlink_blocks(const Geom& g) { return grid_for(g.V, RED_BS, red_cap()); }
int meanlink_slots(const Geom& g) { return grid_for(g.V, RED_BS, kMaxRedBlocks); }

template <typename T, typename G2>
__device__ __forceinline__ M3<T> load_g(const G2* __restrict__ G, int64_t V, int64_t s) {
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
__global__ void __launch_bounds__(RED_BS) k_meanlink(L U, Geom g, const G2* __restrict__ G, double* __restrict__ part) {
    __shared__ double sh[32];
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.V; s += (int64_t)gridDim.x * blockDim.x) {
        int c[4];
        site_coords(g, s, c);
        const M3<T> gx = load_g<T>(G, g.V, s);
#pragma unroll
        for (int mu = 0; mu < 4; ++mu) {
            const M3<T> gp = load_g<T>(G, g.V, s + disp(g, mu, c[mu], 1));
            const M3<T> gu = mul(gx, U.load(s, mu));
            acc[mu] += (double)retr_mm<false, true>(gu, gp);
        }
    }
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
        const double r = block_sum(acc[mu], sh);
        if (threadIdx.x == 0) part[mu * gridDim.x + blockIdx.x] = r;
    }
}

cudaError_t launch_meanlink(const FieldRef& U, const void* G, int g_dtype, double* part, double* out4, cudaStream_t st) {
    const int nb = meanlink_blocks(U.g);
    FLUE_DISPATCH_LINKS(U, {
        if (g_dtype == PREC_C128)
            note_launch(), k_meanlink<decltype(L), T, double2><<<nb, RED_BS, 0, st>>>(L, U.g, (const double2*)G, part);
        else
            note_launch(), k_meanlink<decltype(L), T, float2><<<nb, RED_BS, 0, st>>>(L, U.g, (const float2*)G, part);
    });
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_finish_sums(part, nb, 4, out4, st);
}

FLUE_OOB_READER(observables)

}  // namespace flue
