// ensemble.cu -- plaquette / Polyakov / B^2 of an ensemble of gauge fields of
// uneven volume in ONE persistent launch, replayed from a CUDA graph.
//
// The launch is a dataflow scheduler: a cooperative persistent grid (every
// block resident at once) takes tasks from a global counter in list order.
//   LINES(j, c): the straight lines L^1..3 of the spatial directions for
//                chunk c of time slab j (one block of sites), written into
//                ring slot j % kSlots of the workspace;
//   FWD(j, c):   the 5-loop F of the planes (3,2), (2,4), (4,3) at the sites
//                of chunk c of slab j, built from those lines (84 products
//                per plane-site), and the partial sum of -Re Tr(F F);
//   COLS(f, c):  spatial and temporal plaquettes and the Polyakov loops of a
//                run of time columns of field f.
// FWD(j, .) waits until every LINES(j, .) has finished, and LINES(j, .)
// waits until every FWD(j - kSlots, .) has released the slot.  The list
// places LINES(j) before FWD(j - 1), so every task waits only on tasks with
// lower indices: those were taken by resident blocks and finish, so the
// schedule always progresses.  Every wait is bounded; a wait that runs out
// sets an error flag (the call then reports FLUE_ERR_TIMEOUT), and the
// other waits give up as soon as they see it.  Each task writes its own FP64
// partials; a finisher sums each field's partials in list order, so results
// do not depend on which block took which task.
//
// Per site: spatial and temporal plaquettes (src/wloops.F90:915-1017), the
// 5-loop B^2 integrand -Re Tr(F F) of the planes (3,2),(2,4),(4,3)
// (src/wloops.F90:479-544), and per column the Polyakov loop
// (src/wloops.F90:1019-1069).
//
// Output per field (6 doubles): [sum Re Tr P spatial, sum Re Tr P temporal,
// sum Re Tr Polyakov, sum Im Tr Polyakov, B^2 (already divided by V), V].
#include <stdlib.h>

#include <mutex>
#include <vector>

#include "../../include/flue_gb300.h"
#include "flue_internal.h"
#include "loop5.cuh"

namespace flue {

constexpr int NOBS = 6;

struct EnsField {
    const void* links;
    Geom g;
};

enum EnsTaskType : int { TASK_LINES = 0, TASK_FWD = 1, TASK_COLS = 2 };

struct EnsTask {
    int type;
    int a;  // LINES / FWD: slab; COLS: field
    int b;  // LINES / FWD: chunk (block-sized run of the slab's sites); COLS: first column
    int n;  // COLS: number of columns
};

// A time slab: the time slices [t0, t0 + nts) of one field, as a lattice of
// its own (time extent nts); B^2 never steps in time, so slabs are
// independent.
struct EnsSlab {
    int field, t0, nts, nchunk;
};

// ring slots of slab lines
constexpr int kSlots = 4;
// sites per slab aimed at (whole time slices): 2^17, as the device B^2, or
// FLUE_ENS_SLAB_SITES (read when an ensemble is created; small values make
// many slabs, which the tests use to exercise the ring)
static int64_t slab_sites() {
    const char* env = getenv("FLUE_ENS_SLAB_SITES");
    const long long v = env ? atoll(env) : 0;
    if (v <= 0) return (int64_t)1 << 17;
    return v > ((long long)1 << 22) ? (int64_t)1 << 22 : (int64_t)v;
}

struct EnsFlowArgs {
    const EnsField* fields;
    const EnsSlab* slabs;
    const EnsTask* tasks;
    int ntasks, nslabs;
    int* ctr;      // [0] task counter, [1] error flag, [2, 2 + nslabs) lines done, then fwd done
    double* part;  // NOBS per task
    char* ring;    // kSlots slots of slot_bytes
    size_t slot_bytes;
    PlaneArg pa;   // the B^2 planes
};

// Thread 0: wait until *p >= target, at most ~1.7 s; false (and the error
// flag set) when the wait runs out or another wait already failed.
__device__ __forceinline__ bool flow_wait(const int* p, int target, int* err) {
    for (int it = 0; it < (1 << 24); ++it) {
        int v;
        asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
        if (v >= target) {
            __threadfence();
            return true;
        }
        if ((it & 255) == 255 && *(volatile int*)err) return false;
        __nanosleep(100);
    }
    atomicExch(err, 1);
    return false;
}

// link accessor of a field's pointer in the precision L reads
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

// FP32: registers capped for 12 resident warps per SM (the forward kernel's
// budget); FP64 keeps what it needs (bound by the FP64 pipe)
template <typename T, int BS>
struct FlowMinBlocks {
    static constexpr int value = 1;
};
template <>
struct FlowMinBlocks<float, 128> {
    static constexpr int value = 3;
};
template <class L, typename T, int BS>
__global__ void __launch_bounds__(BS, (FlowMinBlocks<T, BS>::value)) k_ens_flow(EnsFlowArgs a) {
    __shared__ double sh[32];
    __shared__ int cur, ok;
    int* const err = a.ctr + 1;
    int* const lines_done = a.ctr + 2;
    int* const fwd_done = a.ctr + 2 + a.nslabs;
    // every task is taken once: at most ntasks + 1 turns per block
    for (int guard = 0; guard <= a.ntasks; ++guard) {
        if (threadIdx.x == 0) cur = atomicAdd(a.ctr, 1);
        __syncthreads();
        const int t = cur;
        if (t >= a.ntasks) break;
        const EnsTask tk = a.tasks[t];
        if (tk.type == TASK_COLS) {
            const EnsField f = a.fields[tk.a];
            const L U = LinksFrom<L>::make(f.links, f.g.V);
            const int nt = f.g.n[0];
            double sp = 0.0, tp = 0.0, pr = 0.0, pi = 0.0;
            const int nsites = tk.n * nt;
            for (int k = threadIdx.x; k < nsites; k += BS) {
                const int64_t s = (int64_t)tk.b * nt + k;
                int c[4];
                site_coords(f.g, s, c);
                plaq_site<L, T>(U, f.g, s, c, sp, tp);
            }
            for (int col = threadIdx.x; col < tk.n; col += BS) {
                const int64_t s0 = (int64_t)(tk.b + col) * nt;
                M3<T> pl = U.load(s0, 0);
                for (int tt = 1; tt < nt; ++tt) pl = mul(pl, U.load(s0 + tt, 0));
                pr += (double)retr(pl);
                pi += (double)(pl.i[0] + pl.i[4] + pl.i[8]);
            }
            const double v[4] = {sp, tp, pr, pi};
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const double r = block_sum(v[o], sh);
                if (threadIdx.x == 0) a.part[(int64_t)t * NOBS + o] = r;
            }
        } else {
            const int j = tk.a;
            const EnsSlab sl = a.slabs[j];
            const EnsField f = a.fields[sl.field];
            const Geom g = make_geom(sl.nts, f.g.n[1], f.g.n[2], f.g.n[3]);
            using VP = decltype(MatAoS<T>::p);
            const MatAoS<T> lines{reinterpret_cast<VP>(a.ring + (size_t)(j % kSlots) * a.slot_bytes), g.V};
            const int64_t s = (int64_t)tk.b * BS + threadIdx.x;
            if (tk.type == TASK_LINES) {
                // the slot is free once every FWD task of slab j - kSlots is done
                if (threadIdx.x == 0)
                    ok = j < kSlots || flow_wait(fwd_done + (j - kSlots), a.slabs[j - kSlots].nchunk, err);
                __syncthreads();
                if (ok && s < g.V) {
                    const L U = LinksFrom<L>::make(f.links, f.g.V);
#pragma unroll 1
                    for (int slot = 0; slot < a.pa.nd; ++slot) line_site<L, T>(U, g, f.g, sl.t0, a.pa, lines, s, slot);
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    __threadfence();
                    atomicAdd(lines_done + j, 1);
                }
            } else {
                if (threadIdx.x == 0) ok = flow_wait(lines_done + j, sl.nchunk, err);
                __syncthreads();
                double e = 0.0;
                if (ok && s < g.V) {
                    int c[4];
                    site_coords(g, s, c);
#pragma unroll 1
                    for (int p = 0; p < a.pa.np; ++p) {
                        const M3<T> fm = ah_quarter(fwd_q<T, uint32_t>(g, a.pa, 1, lines, s, c, p));
                        e -= (double)retr_mm<false, false>(fm, fm);
                    }
                }
                const double r = block_sum(e, sh);
                if (threadIdx.x == 0) {
                    a.part[(int64_t)t * NOBS + 4] = r;
                    __threadfence();
                    atomicAdd(fwd_done + j, 1);
                }
            }
        }
        __syncthreads();
    }
}

// out[f*NOBS + o] = sum of the field's task partials in list order (its
// tasks are ftask[ffirst[f] .. ffirst[f+1])); B^2 divided by V.  When a wait
// of the scheduler ran out (err != 0) every observable is NaN.
__global__ void k_ensemble_finish(const double* __restrict__ part, const int* __restrict__ ffirst,
                                  const int* __restrict__ ftask, const EnsField* fields, int nfields,
                                  const int* __restrict__ err, double* __restrict__ out) {
    const int f = blockIdx.x;
    if (f >= nfields) return;
    const int o = threadIdx.x;
    if (o >= NOBS) return;
    if (o == 5) {
        out[f * NOBS + 5] = (double)fields[f].g.V;
        return;
    }
    double acc = 0.0;
    for (int k = ffirst[f]; k < ffirst[f + 1]; ++k) acc += part[(int64_t)ftask[k] * NOBS + o];
    if (o == 4) acc /= (double)fields[f].g.V;
    out[f * NOBS + o] = *err ? __longlong_as_double(0x7ff8000000000000LL) : acc;
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
    int ntasks = 0;
    int nslabs = 0;
    int tile = 0;
    int grid = 0;
    int block = 128;
    int with_b2 = 1;
    EnsField* d_fields = nullptr;
    EnsSlab* d_slabs = nullptr;
    EnsTask* d_tasks = nullptr;
    int* d_ffirst = nullptr;
    int* d_ftask = nullptr;
    int* d_ctr = nullptr;  // task counter, error flag, per-slab done counters
    double* d_part = nullptr;
    char* d_ring = nullptr;
    size_t slot_bytes = 0;
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

template <class L, typename T, int BS>
static cudaError_t flow_launch(const EnsFlowArgs& args, int grid, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(BS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // every block resident: the waits in the kernel progress
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    note_launch();
    return cudaLaunchKernelEx(&cfg, k_ens_flow<L, T, BS>, args);
}

template <int BS>
static cudaError_t flow_dispatch(const flue_ensemble* e, const EnsFlowArgs& args, cudaStream_t st) {
    if (e->prec == PREC_C128) return flow_launch<FullLinks<double>, double, BS>(args, e->grid, st);
    if (e->prec == PREC_C64) return flow_launch<FullLinks<float>, float, BS>(args, e->grid, st);
    return flow_launch<R12Links, float, BS>(args, e->grid, st);
}

static PlaneArg b2_plane_arg() {
    // magnetic: Loop5(3,2), Loop5(2,4), Loop5(4,3) (src/wloops.F90:502-506), 0-based
    PlaneArg pa;
    pa.np = 3;
    const int mu[3] = {2, 1, 3}, nu[3] = {1, 3, 2};
    for (int k = 0; k < 4; ++k) pa.slot[k] = -1, pa.dir[k] = -1;
    pa.nd = 0;
    for (int p = 0; p < 3; ++p) {
        pa.mu[p] = mu[p];
        pa.nu[p] = nu[p];
        for (int d : {mu[p], nu[p]})
            if (pa.slot[d] < 0) pa.slot[d] = pa.nd, pa.dir[pa.nd++] = d;
    }
    for (int p = 3; p < 6; ++p) pa.mu[p] = pa.nu[p] = 0;
    return pa;
}

static cudaError_t ens_launch(flue_ensemble* e, double* d_out, cudaStream_t st) {
    if (e->pipeline) return ens_launch_pipeline(e, d_out, st);
    cudaError_t r = cudaMemsetAsync(e->d_ctr, 0, sizeof(int) * (2 + 2 * (size_t)e->nslabs), st);
    if (r != cudaSuccess) return r;
    EnsFlowArgs args;
    args.fields = e->d_fields;
    args.slabs = e->d_slabs;
    args.tasks = e->d_tasks;
    args.ntasks = e->ntasks;
    args.nslabs = e->nslabs;
    args.ctr = e->d_ctr;
    args.part = e->d_part;
    args.ring = e->d_ring;
    args.slot_bytes = e->slot_bytes;
    args.pa = b2_plane_arg();
    r = e->block == 256 ? flow_dispatch<256>(e, args, st) : flow_dispatch<128>(e, args, st);
    if (r != cudaSuccess) return r;
    note_launch(), k_ensemble_finish<<<e->nfields, 32, 0, st>>>(e->d_part, e->d_ffirst, e->d_ftask, e->d_fields,
                                                               e->nfields, e->d_ctr + 1, d_out);
    return cudaGetLastError();
}

static void ens_free(flue_ensemble* e) {
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    cudaFree(e->d_fields);
    cudaFree(e->d_slabs);
    cudaFree(e->d_tasks);
    cudaFree(e->d_ffirst);
    cudaFree(e->d_ftask);
    cudaFree(e->d_ctr);
    cudaFree(e->d_part);
    cudaFree(e->d_ring);
    cudaFree(e->d_ws);
    delete e;
}

template <class L, typename T, int BS>
static int flow_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_ens_flow<L, T, BS>, BS, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

static int flow_occupancy(int prec, int block) {
    if (block == 256) {
        if (prec == PREC_C128) return flow_blocks_per_sm<FullLinks<double>, double, 256>();
        if (prec == PREC_C64) return flow_blocks_per_sm<FullLinks<float>, float, 256>();
        return flow_blocks_per_sm<R12Links, float, 256>();
    }
    if (prec == PREC_C128) return flow_blocks_per_sm<FullLinks<double>, double, 128>();
    if (prec == PREC_C64) return flow_blocks_per_sm<FullLinks<float>, float, 128>();
    return flow_blocks_per_sm<R12Links, float, 128>();
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
    for (int f = 0; f < nfields; ++f) {
        const flue_field& F = fields[f];
        if (!F.links) return FLUE_ERR_ARG;
        if (F.prec != prec) return FLUE_ERR_DTYPE;  // one precision per ensemble
        if (F.prec != FLUE_C128 && F.prec != FLUE_C64 && F.prec != FLUE_R12) return FLUE_ERR_DTYPE;
        if (F.nt < 1 || F.nx < 1 || F.ny < 1 || F.nz < 1 || (int64_t)F.nt * F.nx * F.ny * F.nz >= ((int64_t)1 << 31))
            return FLUE_ERR_SHAPE;
        hf[f].links = F.links;
        hf[f].g = make_geom(F.nt, F.nx, F.ny, F.nz);
    }
    // the task list (see the top of the file): per slab j its LINES tasks,
    // then the FWD tasks of slab j - 1; the COLS tasks last
    std::vector<EnsSlab> slabs;
    std::vector<EnsTask> tasks;
    std::vector<std::vector<int>> per_field(nfields);
    int64_t max_slab = 1;
    if (!pipeline) {
        for (int f = 0; f < nfields && with_b2; ++f) {
            const Geom& g = hf[f].g;
            const int64_t v3 = g.V / g.n[0];
            const int64_t want = slab_sites();
            int nts = (int)((want + v3 - 1) / v3);
            if (nts > g.n[0]) nts = g.n[0];
            if (nts < 1) nts = 1;
            for (int t0 = 0; t0 < g.n[0]; t0 += nts) {
                const int n = g.n[0] - t0 < nts ? g.n[0] - t0 : nts;
                const int64_t vs = (int64_t)n * v3;
                // the forward reads a slab's lines with 32-bit offsets
                if (!(prec == FLUE_C128 ? MatAoS<double>::fits32(vs, 9) : MatAoS<float>::fits32(vs, 9)))
                    return FLUE_ERR_SHAPE;
                if (vs > max_slab) max_slab = vs;
                slabs.push_back({f, t0, n, (int)((vs + block - 1) / block)});
            }
        }
        const int ns = (int)slabs.size();
        for (int j = 0; j <= ns; ++j) {
            if (j < ns)
                for (int c = 0; c < slabs[j].nchunk; ++c) tasks.push_back({TASK_LINES, j, c, 0});
            if (j >= 1)
                for (int c = 0; c < slabs[j - 1].nchunk; ++c) {
                    per_field[slabs[j - 1].field].push_back((int)tasks.size());
                    tasks.push_back({TASK_FWD, j - 1, c, 0});
                }
        }
        for (int f = 0; f < nfields; ++f) {
            const int ncol = fields[f].nx * fields[f].ny * fields[f].nz;
            for (int c0 = 0; c0 < ncol; c0 += tile_cols) {
                per_field[f].push_back((int)tasks.size());
                tasks.push_back({TASK_COLS, f, c0, std::min(tile_cols, ncol - c0)});
            }
        }
    }
    std::vector<int> ffirst(nfields + 1, 0), ftask;
    for (int f = 0; f < nfields; ++f) {
        ffirst[f] = (int)ftask.size();
        ftask.insert(ftask.end(), per_field[f].begin(), per_field[f].end());
    }
    ffirst[nfields] = (int)ftask.size();
    if (ftask.empty()) ftask.push_back(0);  // (keeps the allocations non-empty)
    if (slabs.empty()) slabs.push_back({0, 0, 1, 0});
    if (tasks.empty()) tasks.push_back({TASK_COLS, 0, 0, 0});
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    flue_ensemble* e = new flue_ensemble();
    e->prec = prec;
    e->nfields = nfields;
    e->tile = tile_cols;
    e->block = block;
    e->with_b2 = with_b2 ? 1 : 0;
    cudaError_t r = cudaSuccess;
    if (pipeline) {
        e->pipeline = 1;
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
    } else {
        // every block must be resident (cooperative launch)
        const int occ = flow_occupancy(prec, block);
        if (occ < 1) {
            ens_free(e);
            return FLUE_ERR_CUDA;
        }
        e->grid = nsm * (blocks_per_sm < occ ? blocks_per_sm : occ);
        e->ntasks = (int)tasks.size();
        e->nslabs = (int)slabs.size();
        e->slot_bytes = (prec == PREC_C128 ? MatAoS<double>::bytes(max_slab, 9) : MatAoS<float>::bytes(max_slab, 9));
        e->slot_bytes = (e->slot_bytes + 255) & ~(size_t)255;
        if ((r = cudaMalloc(&e->d_ring, kSlots * e->slot_bytes)) != cudaSuccess) {
            ens_free(e);
            cudaGetLastError();
            return FLUE_ERR_NOMEM;
        }
    }
    if ((r = cudaMalloc(&e->d_fields, sizeof(EnsField) * nfields)) != cudaSuccess ||
        (r = cudaMalloc(&e->d_slabs, sizeof(EnsSlab) * slabs.size())) != cudaSuccess ||
        (r = cudaMalloc(&e->d_tasks, sizeof(EnsTask) * tasks.size())) != cudaSuccess ||
        (r = cudaMalloc(&e->d_ffirst, sizeof(int) * (nfields + 1))) != cudaSuccess ||
        (r = cudaMalloc(&e->d_ftask, sizeof(int) * ftask.size())) != cudaSuccess ||
        (r = cudaMalloc(&e->d_ctr, sizeof(int) * (2 + 2 * slabs.size()))) != cudaSuccess ||
        (r = cudaMalloc(&e->d_part, sizeof(double) * NOBS * tasks.size())) != cudaSuccess) {
        ens_free(e);
        cudaGetLastError();
        return FLUE_ERR_NOMEM;
    }
    if ((r = cudaMemcpy(e->d_fields, hf.data(), sizeof(EnsField) * nfields, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (r = cudaMemcpy(e->d_slabs, slabs.data(), sizeof(EnsSlab) * slabs.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (r = cudaMemcpy(e->d_tasks, tasks.data(), sizeof(EnsTask) * tasks.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (r = cudaMemcpy(e->d_ffirst, ffirst.data(), sizeof(int) * (nfields + 1), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (r = cudaMemcpy(e->d_ftask, ftask.data(), sizeof(int) * ftask.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (r = cudaMemset(e->d_part, 0, sizeof(double) * NOBS * tasks.size())) != cudaSuccess) {
        ens_free(e);
        return FLUE_ERR_CUDA;
    }
    *out = e;
    return FLUE_OK;
}

int flue_ensemble_items(const flue_ensemble* e) { return e ? e->ntasks : -1; }

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
