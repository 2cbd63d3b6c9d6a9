// ensemble.cu -- plaquette / Polyakov / B^2 of an ensemble of gauge fields of
// uneven volume in ONE persistent launch, replayed from a CUDA graph.
//
// Work list: every field is cut into items of `tile` complete time columns
// (a column = the NT sites of one spatial site), so that an item can also
// form the Polyakov loops of its columns.  A persistent grid (a multiple of
// the SM count) takes items from a global counter with atomicAdd -- no block
// ever waits on another, so nothing can hang -- and writes one FP64 partial
// per observable and item.  A finisher sums each field's items in item order,
// so results do not depend on which block took which item.
//
// Per site: spatial and temporal plaquettes (src/wloops.F90:915-1017), the
// 5-loop B^2 integrand -Re Tr(F F) of the planes (3,2),(2,4),(4,3)
// (src/wloops.F90:479-544) with every leaf walked link by link (no scratch
// intermediates; 180 products per plane), and per column the Polyakov loop
// (src/wloops.F90:1019-1069).
//
// Output per field (6 doubles): [sum Re Tr P spatial, sum Re Tr P temporal,
// sum Re Tr Polyakov, sum Im Tr Polyakov, B^2 (already divided by V), V].
#include <mutex>
#include <vector>

#include "../../include/flue_gb300.h"
#include "flue_internal.h"

namespace flue {

constexpr int NOBS = 6;

struct EnsField {
    const void* links;
    Geom g;
};

struct EnsItem {
    int field;
    int col0;   // first spatial site (column) of the item
    int ncols;  // columns in the item
};

// 28 leaves of one plane as path steps in units of (mu, nu): +1/-1 = +-mu,
// +2/-2 = +-nu (src/wloops.F90:236-290), with the weight of their shape.
struct LeafTable {
    int n;           // number of leaves
    int len[28];     // steps of leaf l
    int off[28];     // first step of leaf l in `step`
    double wgt[28];  // weight (k1, k2, k5, k3/2, k4/2)
    signed char step[208];
};

__constant__ LeafTable c_leaves;

static void build_leaf_table(LeafTable* t) {
    const double k5 = 1.0 / 180.0, k1 = (19.0 / 9.0) - 55.0 * k5, k2 = (1.0 / 36.0) - 16.0 * k5,
                 k3 = 64.0 * k5 - (32.0 / 45.0), k4 = (1.0 / 15.0) - 6.0 * k5;
    struct Sh {
        int a, b;
        double w;
    } sh[7] = {{1, 1, k1}, {2, 2, k2}, {3, 3, k5}, {1, 2, 0.5 * k3}, {2, 1, 0.5 * k3}, {1, 3, 0.5 * k4}, {3, 1, 0.5 * k4}};
    int nl = 0, ns = 0;
    for (auto& s : sh) {
        // the four counter-clockwise leaves of the a x b rectangles with the
        // site as corner: (mu^a nu^b -mu^a -nu^b), (nu^b -mu^a -nu^b mu^a), ...
        const int seg[4][4] = {{1, 2, -1, -2}, {2, -1, -2, 1}, {-1, -2, 1, 2}, {-2, 1, 2, -1}};
        for (int q = 0; q < 4; ++q) {
            t->off[nl] = ns;
            t->wgt[nl] = s.w;
            for (int e = 0; e < 4; ++e) {
                const int dir = seg[q][e];
                const int rep = (dir == 1 || dir == -1) ? s.a : s.b;
                for (int r = 0; r < rep; ++r) t->step[ns++] = (signed char)dir;
            }
            t->len[nl] = ns - t->off[nl];
            ++nl;
        }
    }
    t->n = nl;
}

template <class L>
struct LinksFrom;
template <>
struct LinksFrom<FullLinks<double>> {
    __device__ static FullLinks<double> make(const void* p, int64_t V) { return {(const double2*)p, V}; }
};
template <>
struct LinksFrom<FullLinks<float>> {
    __device__ static FullLinks<float> make(const void* p, int64_t V) { return {(const float2*)p, V}; }
};
template <>
struct LinksFrom<R12Links> {
    __device__ static R12Links make(const void* p, int64_t V) { return {(const float4*)p, V}; }
};

template <class L, typename T>
__device__ __forceinline__ M3<T> walk_leaf(const L& U, const Geom& g, int64_t s, const int c[4], int mu, int nu, int l) {
    int cm = 0, cn = 0, nm = 1, nn = 1;
    int64_t stm = 0, stn = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        if (d == mu) cm = c[d], nm = g.n[d], stm = g.st[d];
        if (d == nu) cn = c[d], nn = g.n[d], stn = g.st[d];
    }
    int64_t site = s;
    M3<T> p = m_ident<T>();
    const int o = c_leaves.off[l], n = c_leaves.len[l];
    for (int k = 0; k < n; ++k) {
        const int st = c_leaves.step[o + k];
        const bool along_mu = (st == 1 || st == -1);
        const int dir = along_mu ? mu : nu;
        if (st > 0) {
            p = mul(p, U.load(site, dir));
            if (along_mu) {
                const int nc = cm + 1 == nm ? 0 : cm + 1;
                site += (int64_t)(nc - cm) * stm;
                cm = nc;
            } else {
                const int nc = cn + 1 == nn ? 0 : cn + 1;
                site += (int64_t)(nc - cn) * stn;
                cn = nc;
            }
        } else {
            if (along_mu) {
                const int nc = cm == 0 ? nm - 1 : cm - 1;
                site += (int64_t)(nc - cm) * stm;
                cm = nc;
            } else {
                const int nc = cn == 0 ? nn - 1 : cn - 1;
                site += (int64_t)(nc - cn) * stn;
                cn = nc;
            }
            p = mm<false, true>(p, U.load(site, dir));
        }
    }
    return p;
}

template <class L, typename T>
__device__ double b2_site(const L& U, const Geom& g, int64_t s, const int c[4]) {
    // planes (3,2),(2,4),(4,3) 1-based -> (2,1),(1,3),(3,2) 0-based
    double acc = 0.0;
#pragma unroll 1
    for (int p = 0; p < 3; ++p) {
        const int pmu = p == 0 ? 2 : (p == 1 ? 1 : 3), pnu = p == 0 ? 1 : (p == 1 ? 3 : 2);
        M3<T> q = m_zero<T>();
#pragma unroll 1
        for (int l = 0; l < c_leaves.n; ++l) {
            const M3<T> w = walk_leaf<L, T>(U, g, s, c, pmu, pnu, l);
            m_axpy(q, (T)c_leaves.wgt[l], w);
        }
        const M3<T> f = ah_quarter(q);
        acc -= (double)retr_mm<false, false>(f, f);
    }
    return acc;
}

template <class L, typename T>
__device__ __forceinline__ void plaq_site(const L& U, const Geom& g, int64_t s, const int c[4], double& sp, double& tp) {
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
        const int64_t smu = s + disp(g, mu, c[mu], 1);
        const M3<T> umu = U.load(s, mu);
#pragma unroll
        for (int nu = mu + 1; nu < 4; ++nu) {
            const int64_t snu = s + disp(g, nu, c[nu], 1);
            const M3<T> a = mul(umu, U.load(smu, nu));
            const M3<T> b = mul(U.load(s, nu), U.load(snu, mu));
            const double v = (double)retr_mm<false, true>(a, b);
            if (mu == 0)
                tp += v;
            else
                sp += v;
        }
    }
}

template <class L, typename T>
__global__ void __launch_bounds__(256) k_ensemble(const EnsField* __restrict__ fields, const EnsItem* __restrict__ items,
                                                  int nitems, int* __restrict__ counter, double* __restrict__ part,
                                                  int with_b2) {
    __shared__ double sh[32];
    __shared__ int cur;
    // persistent loop; at most nitems + gridDim.x iterations in total
    for (int guard = 0; guard <= nitems; ++guard) {
        if (threadIdx.x == 0) cur = atomicAdd(counter, 1);
        __syncthreads();
        const int it = cur;
        if (it >= nitems) break;
        const EnsItem item = items[it];
        const EnsField f = fields[item.field];
        const L U = LinksFrom<L>::make(f.links, f.g.V);
        const int nt = f.g.n[0];
        double sp = 0.0, tp = 0.0, pr = 0.0, pi = 0.0, b2 = 0.0;
        const int nsites = item.ncols * nt;
        for (int k = threadIdx.x; k < nsites; k += blockDim.x) {
            const int64_t s = (int64_t)item.col0 * nt + k;
            int c[4];
            site_coords(f.g, s, c);
            plaq_site<L, T>(U, f.g, s, c, sp, tp);
            if (with_b2) b2 += b2_site<L, T>(U, f.g, s, c);
        }
        for (int col = threadIdx.x; col < item.ncols; col += blockDim.x) {
            const int64_t s0 = (int64_t)(item.col0 + col) * nt;
            M3<T> p = U.load(s0, 0);
            for (int t = 1; t < nt; ++t) p = mul(p, U.load(s0 + t, 0));
            pr += (double)retr(p);
            pi += (double)(p.i[0] + p.i[4] + p.i[8]);
        }
        double v[5] = {sp, tp, pr, pi, b2};
#pragma unroll
        for (int o = 0; o < 5; ++o) {
            const double r = block_sum(v[o], sh);
            if (threadIdx.x == 0) part[(int64_t)it * NOBS + o] = r;
        }
        __syncthreads();
    }
}

// out[f*NOBS + o] = sum over the field's items, in order; B^2 divided by V.
__global__ void k_ensemble_finish(const double* __restrict__ part, const int* __restrict__ first, const EnsField* fields,
                                  int nfields, double* __restrict__ out) {
    const int f = blockIdx.x;
    if (f >= nfields) return;
    const int o = threadIdx.x;
    if (o >= NOBS) return;
    if (o == 5) {
        out[f * NOBS + 5] = (double)fields[f].g.V;
        return;
    }
    double acc = 0.0;
    for (int it = first[f]; it < first[f + 1]; ++it) acc += part[(int64_t)it * NOBS + o];
    if (o == 4) acc /= (double)fields[f].g.V;
    out[f * NOBS + o] = acc;
}

FLUE_OOB_READER(ensemble)

}  // namespace flue

// ===========================================================================
// C ABI
// ===========================================================================
using namespace flue;

struct flue_ensemble {
    int prec = 0;
    int nfields = 0;
    int nitems = 0;
    int tile = 0;
    int grid = 0;
    int block = 256;
    int with_b2 = 1;
    EnsField* d_fields = nullptr;
    EnsItem* d_items = nullptr;
    int* d_first = nullptr;
    int* d_counter = nullptr;
    double* d_part = nullptr;
    double* d_out = nullptr;  // output the graph writes to
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // pipeline mode (tile_cols = 0): per field the device entry points
    // (plaquettes, Polyakov loop, line-based B^2) with one library workspace
    int pipeline = 0;
    std::vector<flue_field> hfields;
    void* d_ws = nullptr;
    size_t ws_bytes = 0;
    uint64_t launches_per_eval = 2;  // kernels one replay runs
};

static std::once_flag g_leaf_once;
static cudaError_t g_leaf_err = cudaSuccess;

static cudaError_t ensure_leaf_table() {
    std::call_once(g_leaf_once, [] {
        LeafTable t;
        build_leaf_table(&t);
        g_leaf_err = cudaMemcpyToSymbol(c_leaves, &t, sizeof(t));
    });
    return g_leaf_err;
}

// V of every field (and B^2 = 0 without it) into the output of pipeline mode
__global__ void k_ensemble_volumes(const EnsField* __restrict__ fields, int nfields, int with_b2,
                                   double* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfields) return;
    out[f * NOBS + 5] = (double)fields[f].g.V;
    if (!with_b2) out[f * NOBS + 4] = 0.0;
}

static cudaError_t ens_launch_pipeline(flue_ensemble* e, double* d_out, cudaStream_t st) {
    for (int f = 0; f < e->nfields; ++f) {
        const flue_field* U = &e->hfields[f];
        double* o = d_out + (size_t)f * NOBS;
        int rc = flue_plaquette(U, 2, 4, 4, o, e->d_ws, e->ws_bytes, st);  // spatial planes
        if (!rc) rc = flue_plaquette(U, 1, 1, 4, o + 1, e->d_ws, e->ws_bytes, st);  // temporal planes
        if (!rc) rc = flue_polyakov(U, o + 2, e->d_ws, e->ws_bytes, st);
        if (!rc && e->with_b2) rc = flue_magnetic(U, o + 4, e->d_ws, e->ws_bytes, st);
        if (rc) return cudaErrorUnknown;
    }
    note_launch(), k_ensemble_volumes<<<(e->nfields + 127) / 128, 128, 0, st>>>(e->d_fields, e->nfields, e->with_b2,
                                                                                d_out);
    return cudaGetLastError();
}

static cudaError_t ens_launch(flue_ensemble* e, double* d_out, cudaStream_t st) {
    if (e->pipeline) return ens_launch_pipeline(e, d_out, st);
    cudaError_t r = cudaMemsetAsync(e->d_counter, 0, sizeof(int), st);
    if (r != cudaSuccess) return r;
    if (e->prec == PREC_C128)
        note_launch(), k_ensemble<FullLinks<double>, double>
            <<<e->grid, e->block, 0, st>>>(e->d_fields, e->d_items, e->nitems, e->d_counter, e->d_part, e->with_b2);
    else if (e->prec == PREC_C64)
        note_launch(), k_ensemble<FullLinks<float>, float>
            <<<e->grid, e->block, 0, st>>>(e->d_fields, e->d_items, e->nitems, e->d_counter, e->d_part, e->with_b2);
    else
        note_launch(), k_ensemble<R12Links, float>
            <<<e->grid, e->block, 0, st>>>(e->d_fields, e->d_items, e->nitems, e->d_counter, e->d_part, e->with_b2);
    r = cudaGetLastError();
    if (r != cudaSuccess) return r;
    note_launch(), k_ensemble_finish<<<e->nfields, 32, 0, st>>>(e->d_part, e->d_first, e->d_fields, e->nfields, d_out);
    return cudaGetLastError();
}

static void ens_free(flue_ensemble* e) {
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    cudaFree(e->d_fields);
    cudaFree(e->d_items);
    cudaFree(e->d_first);
    cudaFree(e->d_counter);
    cudaFree(e->d_part);
    cudaFree(e->d_ws);
    delete e;
}

extern "C" {

int flue_ensemble_create(flue_ensemble** out, const flue_field* fields, int nfields, int tile_cols, int block,
                         int blocks_per_sm, int with_b2) {
    if (!out || !fields || nfields < 1) return FLUE_ERR_ARG;
    const bool pipeline = tile_cols == 0;
    if (tile_cols < 0 || (!pipeline && ((block != 128 && block != 256) || blocks_per_sm < 1 || blocks_per_sm > 16)))
        return FLUE_ERR_ARG;
    const int prec = fields[0].prec;
    std::vector<EnsField> hf(nfields);
    std::vector<EnsItem> items;
    std::vector<int> first(nfields + 1);
    for (int f = 0; f < nfields; ++f) {
        const flue_field& F = fields[f];
        if (!F.links) return FLUE_ERR_ARG;
        if (F.prec != prec) return FLUE_ERR_DTYPE;  // one precision per ensemble
        if (F.prec != FLUE_C128 && F.prec != FLUE_C64 && F.prec != FLUE_R12) return FLUE_ERR_DTYPE;
        if (F.nt < 1 || F.nx < 1 || F.ny < 1 || F.nz < 1 || (int64_t)F.nt * F.nx * F.ny * F.nz >= ((int64_t)1 << 31))
            return FLUE_ERR_SHAPE;
        hf[f].links = F.links;
        hf[f].g = make_geom(F.nt, F.nx, F.ny, F.nz);
        first[f] = (int)items.size();
        const int ncol = F.nx * F.ny * F.nz;
        if (!pipeline)
            for (int c0 = 0; c0 < ncol; c0 += tile_cols) items.push_back({f, c0, std::min(tile_cols, ncol - c0)});
    }
    first[nfields] = (int)items.size();
    if (pipeline) items.push_back({0, 0, 0});  // (unused; keeps the allocations non-empty)
    cudaError_t r = ensure_leaf_table();
    if (r != cudaSuccess) return FLUE_ERR_CUDA;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    flue_ensemble* e = new flue_ensemble();
    e->prec = prec;
    e->nfields = nfields;
    e->nitems = (int)items.size();
    e->tile = tile_cols;
    e->block = block;
    e->with_b2 = with_b2 ? 1 : 0;
    e->grid = nsm * blocks_per_sm;
    if (pipeline) {
        e->pipeline = 1;
        e->nitems = 0;
        e->hfields.assign(fields, fields + nfields);
        for (const flue_field& F : e->hfields)
            for (int op : {FLUE_OP_PLAQUETTE, FLUE_OP_POLYAKOV, FLUE_OP_MAGNETIC}) {
                if (op == FLUE_OP_MAGNETIC && !e->with_b2) continue;
                const size_t n = flue_workspace_bytes(op, F.nt, F.nx, F.ny, F.nz, F.prec);
                if (n > e->ws_bytes) e->ws_bytes = n;
            }
        if ((r = cudaMalloc(&e->d_ws, e->ws_bytes < 256 ? 256 : e->ws_bytes)) != cudaSuccess) {
            ens_free(e);
            cudaGetLastError();
            return FLUE_ERR_NOMEM;
        }
    }
    if ((r = cudaMalloc(&e->d_fields, sizeof(EnsField) * nfields)) != cudaSuccess ||
        (r = cudaMalloc(&e->d_items, sizeof(EnsItem) * items.size())) != cudaSuccess ||
        (r = cudaMalloc(&e->d_first, sizeof(int) * (nfields + 1))) != cudaSuccess ||
        (r = cudaMalloc(&e->d_counter, sizeof(int))) != cudaSuccess ||
        (r = cudaMalloc(&e->d_part, sizeof(double) * NOBS * items.size())) != cudaSuccess) {
        ens_free(e);
        cudaGetLastError();
        return FLUE_ERR_NOMEM;
    }
    if ((r = cudaMemcpy(e->d_fields, hf.data(), sizeof(EnsField) * nfields, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (r = cudaMemcpy(e->d_items, items.data(), sizeof(EnsItem) * items.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (r = cudaMemcpy(e->d_first, first.data(), sizeof(int) * (nfields + 1), cudaMemcpyHostToDevice)) != cudaSuccess) {
        ens_free(e);
        return FLUE_ERR_CUDA;
    }
    *out = e;
    return FLUE_OK;
}

int flue_ensemble_items(const flue_ensemble* e) { return e ? e->nitems : -1; }

// Direct (uncaptured) launch of the memset + persistent kernel + finisher.
int flue_ensemble_run(flue_ensemble* e, double* d_out, void* stream) {
    if (!e || !d_out) return FLUE_ERR_ARG;
    return ens_launch(e, d_out, (cudaStream_t)stream) == cudaSuccess ? FLUE_OK : FLUE_ERR_CUDA;
}

// Capture the launch sequence writing to d_out into a CUDA graph (on a
// private stream) and instantiate it; flue_ensemble_replay then launches it.
int flue_ensemble_capture(flue_ensemble* e, double* d_out) {
    if (!e || !d_out) return FLUE_ERR_ARG;
    cudaStream_t cs;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return FLUE_ERR_CUDA;
    cudaError_t r = cudaSuccess;
    if (e->pipeline) {
        // one uncaptured evaluation first: the entry points set up their
        // library streams and caches on first use, outside the capture
        r = ens_launch(e, d_out, cs);
        if (r == cudaSuccess) r = cudaStreamSynchronize(cs);
    }
    if (r == cudaSuccess) r = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (r == cudaSuccess) {
        // captured launches are counted by note_launch although they do not
        // run here; take them back out and count them at each replay
        const uint64_t n0 = flue_kernel_launches();
        cudaError_t rl = ens_launch(e, d_out, cs);
        const uint64_t n1 = flue_kernel_launches();
        e->launches_per_eval = n1 - n0;
        flue::note_launch(-(int)(n1 - n0));
        cudaGraph_t g = nullptr;
        r = cudaStreamEndCapture(cs, &g);
        if (rl != cudaSuccess) r = rl;
        if (r == cudaSuccess) {
            if (e->exec) cudaGraphExecDestroy(e->exec);
            if (e->graph) cudaGraphDestroy(e->graph);
            e->graph = g;
            r = cudaGraphInstantiate(&e->exec, g, 0);
            e->d_out = d_out;
        } else if (g) {
            cudaGraphDestroy(g);
        }
    }
    cudaStreamDestroy(cs);
    if (r != cudaSuccess) {
        cudaGetLastError();
        return FLUE_ERR_CUDA;
    }
    return FLUE_OK;
}

int flue_ensemble_replay(flue_ensemble* e, void* stream) {
    if (!e || !e->exec) return FLUE_ERR_ARG;
    flue::note_launch((int)e->launches_per_eval);  // the kernels the graph holds
    return cudaGraphLaunch(e->exec, (cudaStream_t)stream) == cudaSuccess ? FLUE_OK : FLUE_ERR_CUDA;
}

int flue_ensemble_destroy(flue_ensemble* e) {
    if (!e) return FLUE_ERR_ARG;
    ens_free(e);
    return FLUE_OK;
}

}  // extern "C"
