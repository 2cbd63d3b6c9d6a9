// capi.cu -- the extern "C" boundary declared in include/flue_gb300.h.
// Validates every argument on the host, maps CUDA errors to status codes
// and never exits or traps.  The host-buffer tier keeps one set of device
// buffers and one stream per device, guarded by a mutex.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/flue_gb300.h"
#include "flue_internal.h"

using namespace flue;

namespace {

thread_local char g_detail[256] = "";

int fail(int code, const char* msg) {
    snprintf(g_detail, sizeof(g_detail), "%s", msg);
    return code;
}

}  // namespace

namespace flue {

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return FLUE_OK;
    snprintf(g_detail, sizeof(g_detail), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    return FLUE_ERR_CUDA;
}

bool dims_ok(int nt, int nx, int ny, int nz) {
    if (nt < 1 || nx < 1 || ny < 1 || nz < 1) return false;
    const int64_t V = (int64_t)nt * nx * ny * nz;
    return V < ((int64_t)1 << 31);  // nP of one plane is a default integer, as in the reference
}
bool prec_ok(int p) { return p == FLUE_C128 || p == FLUE_C64 || p == FLUE_R12; }

int check_field(const flue_field* U, FieldRef* out) {
    if (!U) return fail(FLUE_ERR_ARG, "field descriptor is NULL");
    if (!U->links) return fail(FLUE_ERR_ARG, "field links pointer is NULL");
    if (!prec_ok(U->prec)) return fail(FLUE_ERR_DTYPE, "unknown field precision");
    if (!dims_ok(U->nt, U->nx, U->ny, U->nz)) return fail(FLUE_ERR_SHAPE, "bad lattice extents");
    const uintptr_t align = U->prec == FLUE_C64 ? 8 : 16;
    if (((uintptr_t)U->links) % align) return fail(FLUE_ERR_LAYOUT, "field pointer misaligned");
    out->links = U->links;
    out->g = make_geom(U->nt, U->nx, U->ny, U->nz);
    out->prec = U->prec;
    return FLUE_OK;
}

}  // namespace flue

namespace {

inline size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

PlaneSet b2_planes() {
    // magnetic: Loop5(3,2), Loop5(2,4), Loop5(4,3)  (src/wloops.F90:502-506)
    PlaneSet ps;
    ps.np = 3;
    ps.mu[0] = 2, ps.nu[0] = 1;
    ps.mu[1] = 1, ps.nu[1] = 3;
    ps.mu[2] = 3, ps.nu[2] = 2;
    return ps;
}
PlaneSet all_planes() {
    PlaneSet ps;
    ps.np = 0;
    for (int m = 0; m < 4; ++m)
        for (int n = m + 1; n < 4; ++n) {
            ps.mu[ps.np] = m;
            ps.nu[ps.np] = n;
            ps.np++;
        }
    return ps;
}

size_t ws_bytes_for(int op, const Geom& g, int prec) {
    switch (op) {
        case FLUE_OP_PLAQUETTE:
            return a256((size_t)plaquette_slots(g) * 8);
        case FLUE_OP_POLYAKOV:
            return a256((size_t)polyakov_slots(g) * 16);
        case FLUE_OP_WMUNU:
            return a256((size_t)wloop_slots(g) * 8);
        case FLUE_OP_FMUNU: {
            PlaneSet ps;
            ps.np = 1;
            ps.mu[0] = 0;
            ps.nu[0] = 1;
            return energy_ws_bytes(g, prec, ps, false);
        }
        case FLUE_OP_MAGNETIC:
            return energy_ws_bytes(g, prec, b2_planes(), false);
        case FLUE_OP_MAGNETIC_FORCE:
            return energy_ws_bytes(g, prec, b2_planes(), true);
        case FLUE_OP_ENERGY_FORCE:
            return energy_ws_bytes(g, prec, all_planes(), true);
        case FLUE_OP_PLAQUETTE_FORCE:
            return a256((size_t)plaqforce_blocks(g) * 4 * 8);
        case FLUE_OP_MEANLINK:
            return a256((size_t)meanlink_slots(g) * 4 * 8);
        case FLUE_OP_WFLOW:
            return wflow_ws_bytes(g);
        case FLUE_OP_GLUON_PROP:
            return gluon_prop_ws_bytes(g, prec);
        default:
            return 0;
    }
}

int check_ws(int op, const FieldRef& F, size_t ws_bytes, const void* ws) {
    const size_t need = ws_bytes_for(op, F.g, F.prec);
    if (need && (!ws || ws_bytes < need)) {
        snprintf(g_detail, sizeof(g_detail), "workspace too small: need %zu bytes, got %zu", need, ws_bytes);
        return FLUE_ERR_WORKSPACE;
    }
    if (ws && ((uintptr_t)ws) % 256) return fail(FLUE_ERR_LAYOUT, "workspace must be 256-byte aligned");
    return FLUE_OK;
}

// Time slabs of a device energy evaluation whose planes leave out the time
// direction (B^2): FLUE_SLABS slabs, else slabs of at least 2^17 sites (at
// most 16), on FLUE_SLAB_STREAMS streams (default 4).  Measured on GB300,
// B^2 force at 64x32^3 FP32: one pass 11.5 ms, 16 slabs on 4 streams 10.6 ms.
int device_slabs(const Geom& g, const PlaneSet& ps, int* nstream) {
    for (int p = 0; p < ps.np; ++p)
        if (ps.mu[p] == 0 || ps.nu[p] == 0) return 1;
    const char* env = getenv("FLUE_SLABS");
    int n = env ? atoi(env) : 0;
    if (n <= 0) {
        const int64_t v3 = g.V / g.n[0];
        int nts = 1;
        while ((int64_t)nts * v3 < ((int64_t)1 << 17) && nts < g.n[0]) nts *= 2;
        n = (g.n[0] + nts - 1) / nts;
        if (n > 16) n = 16;
    }
    if (n > g.n[0]) n = g.n[0];
    const char* es = getenv("FLUE_SLAB_STREAMS");
    int k = es ? atoi(es) : 4;
    *nstream = k < 1 ? 1 : (k > 4 ? 4 : k);
    return n < 1 ? 1 : n;
}

int energy_common(const flue_field* U, const PlaneSet& ps, int op, double* d_E, void* d_force, int form, void* ws,
                  size_t ws_bytes, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (form != FLUE_FORCE_LIE && form != FLUE_FORCE_EUCLID) return fail(FLUE_ERR_ARG, "bad force form");
    if (!d_E && !d_force) return fail(FLUE_ERR_ARG, "nothing to compute");
    const size_t need = energy_ws_bytes(F.g, F.prec, ps, d_force != nullptr);
    if (!ws || ws_bytes < need) {
        snprintf(g_detail, sizeof(g_detail), "workspace too small: need %zu bytes, got %zu", need, ws_bytes);
        return FLUE_ERR_WORKSPACE;
    }
    (void)op;
    if (!stage_timing_on()) {
        int nstream = 1;
        const int nslab = device_slabs(F.g, ps, &nstream);
        if (nslab > 1 && ws_bytes >= energy_slabs_ws_bytes(F.g, F.prec, ps, d_force != nullptr, nslab, nstream))
            return cuda_status(
                launch_energy_slabs(F, ps, d_E, d_force, form, ws, ws_bytes, nslab, nstream, (cudaStream_t)stream));
    }
    return cuda_status(launch_energy(F, ps, d_E, d_force, form, ws, ws_bytes, (cudaStream_t)stream));
}

}  // namespace

void flue::set_error_detail(const char* msg) { snprintf(g_detail, sizeof(g_detail), "%s", msg); }

static std::atomic<unsigned long long> g_launches{0};
void flue::note_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

extern "C" {

const char* flue_strerror(int s) {
    switch (s) {
        case FLUE_OK:
            return "ok";
        case FLUE_ERR_ARG:
            return "invalid argument";
        case FLUE_ERR_SHAPE:
            return "invalid lattice shape";
        case FLUE_ERR_DTYPE:
            return "invalid precision / dtype";
        case FLUE_ERR_LAYOUT:
            return "unsupported layout / alignment";
        case FLUE_ERR_CUDA:
            return "CUDA runtime error";
        case FLUE_ERR_TIMEOUT:
            return "bounded device wait timed out";
        case FLUE_ERR_WORKSPACE:
            return "workspace too small";
        case FLUE_ERR_NOMEM:
            return "device allocation failed";
        default:
            return "unknown status";
    }
}

// Detail of the most recent failure on this thread (not part of the
// reference interface; diagnostic only).
const char* flue_last_error_detail(void) { return g_detail; }

int flue_abi_version(void) { return 1; }

int flue_stage_timing(int enable) { return cuda_status(stage_timing_enable(enable)); }

uint64_t flue_kernel_launches(void) { return (uint64_t)g_launches.load(std::memory_order_relaxed); }

int64_t flue_bounds_errors(void) {
    if (!FLUE_BOUNDS_CHECK) return -1;
    const unsigned c[] = {oob_capi(), oob_ensemble(), oob_flow(), oob_force(), oob_noalloc(), oob_observables(),
                          oob_propagator()};
    int64_t n = 0;
    for (unsigned v : c) n += v == 0xffffffffu ? 0 : v;
    return n;
}

int flue_stage_times(double* ms, int max_stages, int* n_stages) {
    if (!ms || !n_stages || max_stages < 0) return fail(FLUE_ERR_ARG, "NULL pointer");
    return cuda_status(stage_times(ms, max_stages, n_stages));
}

int64_t flue_field_bytes(int nt, int nx, int ny, int nz, int prec) {
    if (!dims_ok(nt, nx, ny, nz) || !prec_ok(prec)) return -1;
    const int64_t V = (int64_t)nt * nx * ny * nz;
    if (prec == FLUE_C128) return V * 36 * 16;
    if (prec == FLUE_C64) return V * 36 * 8;
    return V * 12 * 16;
}

size_t flue_workspace_bytes(int op, int nt, int nx, int ny, int nz, int prec) {
    if (!dims_ok(nt, nx, ny, nz) || !prec_ok(prec)) return 0;
    return ws_bytes_for(op, make_geom(nt, nx, ny, nz), prec);
}

int flue_pack_field(const void* src, int src_dtype, const int64_t strides[7], int nt, int nx, int ny, int nz, void* dst,
                    int dst_prec, int reunitarise, void* stream) {
    if (!src || !dst || !strides) return fail(FLUE_ERR_ARG, "NULL pointer");
    if (src_dtype != FLUE_C128 && src_dtype != FLUE_C64) return fail(FLUE_ERR_DTYPE, "source must be c128 or c64");
    if (!prec_ok(dst_prec)) return fail(FLUE_ERR_DTYPE, "bad destination precision");
    if (!dims_ok(nt, nx, ny, nz)) return fail(FLUE_ERR_SHAPE, "bad lattice extents");
    for (int k = 0; k < 7; ++k)
        if (strides[k] < 0) return fail(FLUE_ERR_LAYOUT, "negative strides are not supported");
    const Geom g = make_geom(nt, nx, ny, nz);
    return cuda_status(launch_pack(src, src_dtype, strides, g, dst, dst_prec, reunitarise, (cudaStream_t)stream));
}

int flue_unpack_field(const flue_field* U, void* dst, int dst_dtype, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!dst) return fail(FLUE_ERR_ARG, "NULL destination");
    if (dst_dtype != FLUE_C128 && dst_dtype != FLUE_C64) return fail(FLUE_ERR_DTYPE, "destination must be c128 or c64");
    return cuda_status(launch_unpack(F, dst, dst_dtype, (cudaStream_t)stream));
}

int flue_reunitarise_field(const flue_field* U, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    return cuda_status(launch_fix_field((void*)F.links, F.g, F.prec, (cudaStream_t)stream));
}

int flue_multiplymatmat_batch(const void* left, const void* right, void* out, int64_t n, int dtype, int dagger,
                              void* stream) {
    if (!left || !right || !out) return fail(FLUE_ERR_ARG, "NULL pointer");
    if (n < 0) return fail(FLUE_ERR_SHAPE, "negative count");
    if (dtype != FLUE_C128 && dtype != FLUE_C64) return fail(FLUE_ERR_DTYPE, "dtype must be c128 or c64");
    if (n == 0) return FLUE_OK;
    return cuda_status(launch_matmul_batch(left, right, out, n, dtype, dagger, (cudaStream_t)stream));
}

int flue_plaquette(const flue_field* U, int muStart, int muEnd, int nuEnd, double* d_sum, void* ws, size_t ws_bytes,
                   void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_sum) return fail(FLUE_ERR_ARG, "NULL output");
    if (muStart < 1 || muEnd > 4 || nuEnd > 4 || muStart > muEnd + 1 || nuEnd < 1)
        return fail(FLUE_ERR_ARG, "plane range out of 1..4");
    if ((rc = check_ws(FLUE_OP_PLAQUETTE, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_plaquette(F, muStart - 1, muEnd - 1, nuEnd - 1, (double*)ws, d_sum, (cudaStream_t)stream));
}

size_t flue_wmunu_table_bytes(int nt, int nx, int ny, int nz, int prec, int rmax, int tmax) {
    if (!dims_ok(nt, nx, ny, nz) || !prec_ok(prec) || rmax < 1 || tmax < 1 || rmax > 64 || tmax > 64) return 0;
    return wmunu_table_ws_bytes(make_geom(nt, nx, ny, nz), prec, rmax, tmax);
}

int flue_wmunu_table(const flue_field* U, int mu, int nu, int rmax, int tmax, double* d_out, void* ws,
                     size_t ws_bytes, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_out) return fail(FLUE_ERR_ARG, "NULL output");
    if (mu < 1 || mu > 4 || nu < 1 || nu > 4) return fail(FLUE_ERR_ARG, "direction out of 1..4");
    if (rmax < 1 || tmax < 1 || rmax > 64 || tmax > 64) return fail(FLUE_ERR_ARG, "rmax, tmax must be 1..64");
    const size_t need = wmunu_table_ws_bytes(F.g, F.prec, rmax, tmax);
    if (!ws || ws_bytes < need) {
        snprintf(g_detail, sizeof(g_detail), "workspace too small: need %zu bytes, got %zu", need, ws_bytes);
        return FLUE_ERR_WORKSPACE;
    }
    if (((uintptr_t)ws) % 256) return fail(FLUE_ERR_LAYOUT, "workspace must be 256-byte aligned");
    return cuda_status(launch_wmunu_table(F, mu - 1, nu - 1, rmax, tmax, d_out, ws, (cudaStream_t)stream));
}

int flue_polyakov(const flue_field* U, double* d_sum2, void* ws, size_t ws_bytes, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_sum2) return fail(FLUE_ERR_ARG, "NULL output");
    if ((rc = check_ws(FLUE_OP_POLYAKOV, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_polyakov(F, (double*)ws, d_sum2, (cudaStream_t)stream));
}

int flue_wmunu(const flue_field* U, int tau, int mu, int nu, int nMu, int nNu, double* d_val, void* ws, size_t ws_bytes,
               void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_val) return fail(FLUE_ERR_ARG, "NULL output");
    if (mu < 1 || mu > 4 || nu < 1 || nu > 4) return fail(FLUE_ERR_ARG, "direction out of 1..4");
    if (nMu < 1 || nNu < 1) return fail(FLUE_ERR_ARG, "loop extents must be >= 1");
    if (tau < 0 || tau > U->nt) return fail(FLUE_ERR_ARG, "tau out of 0..NT");
    if ((rc = check_ws(FLUE_OP_WMUNU, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_wloop(F, tau - 1, mu - 1, nu - 1, nMu, nNu, (double*)ws, d_val, (cudaStream_t)stream));
}

int flue_genericpath(const flue_field* U, const int* coordBase, const int* path, int npath, void* d_out, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_out || (!path && npath > 0)) return fail(FLUE_ERR_ARG, "NULL pointer");
    if (npath < 0 || npath > 256) return fail(FLUE_ERR_ARG, "path length must be 0..256");
    for (int k = 0; k < npath; ++k)
        if (path[k] == 0 || path[k] < -4 || path[k] > 4) return fail(FLUE_ERR_ARG, "path entry out of +-1..+-4");
    if (coordBase) {
        const int n[4] = {U->nt, U->nx, U->ny, U->nz};
        for (int k = 0; k < 4; ++k)
            if (coordBase[k] < 1 || coordBase[k] > n[k]) return fail(FLUE_ERR_ARG, "coordBase out of range");
    }
    return cuda_status(launch_genericpath(F, path, npath, coordBase, d_out, (cudaStream_t)stream));
}

int flue_fmunu(const flue_field* U, int kind, int mu, int nu, void* d_out, void* ws, size_t ws_bytes, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_out) return fail(FLUE_ERR_ARG, "NULL output");
    if (kind != FLUE_FMUNU_CLOVER && kind != FLUE_FMUNU_LOOP5) return fail(FLUE_ERR_ARG, "bad F_munu kind");
    if (mu < 1 || mu > 4 || nu < 1 || nu > 4 || mu == nu) return fail(FLUE_ERR_ARG, "bad plane");
    if ((rc = check_ws(FLUE_OP_FMUNU, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_fmunu(F, kind, mu - 1, nu - 1, d_out, ws, ws_bytes, (cudaStream_t)stream));
}

int flue_magnetic(const flue_field* U, double* d_B, void* ws, size_t ws_bytes, void* stream) {
    if (!d_B) return fail(FLUE_ERR_ARG, "NULL output");
    return energy_common(U, b2_planes(), FLUE_OP_MAGNETIC, d_B, nullptr, FLUE_FORCE_LIE, ws, ws_bytes, stream);
}

int flue_magnetic_force(const flue_field* U, double* d_B, void* d_force, int force_form, void* ws, size_t ws_bytes,
                        void* stream) {
    return energy_common(U, b2_planes(), FLUE_OP_MAGNETIC_FORCE, d_B, d_force, force_form, ws, ws_bytes, stream);
}

int flue_loop5_energy_force(const flue_field* U, const int* planes, int nplanes, double* d_E, void* d_force,
                            int force_form, void* ws, size_t ws_bytes, void* stream) {
    if (!planes || nplanes < 1 || nplanes > 6) return fail(FLUE_ERR_ARG, "nplanes must be 1..6");
    PlaneSet ps;
    ps.np = nplanes;
    int seen = 0;
    for (int p = 0; p < nplanes; ++p) {
        const int m = planes[2 * p], n = planes[2 * p + 1];
        if (m < 1 || m > 4 || n < 1 || n > 4 || m == n) return fail(FLUE_ERR_ARG, "bad plane");
        const int lo = m < n ? m : n, hi = m < n ? n : m;
        const int bit = 1 << (lo * 4 + hi);
        if (seen & bit) return fail(FLUE_ERR_ARG, "plane listed twice");
        seen |= bit;
        ps.mu[p] = m - 1;
        ps.nu[p] = n - 1;
    }
    return energy_common(U, ps, FLUE_OP_ENERGY_FORCE, d_E, d_force, force_form, ws, ws_bytes, stream);
}

int flue_plaquette_force(const flue_field* U, double* d_S, void* d_force, int force_form, void* ws, size_t ws_bytes,
                         void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_S && !d_force) return fail(FLUE_ERR_ARG, "nothing to compute");
    if (force_form != FLUE_FORCE_LIE && force_form != FLUE_FORCE_EUCLID) return fail(FLUE_ERR_ARG, "bad force form");
    if ((rc = check_ws(FLUE_OP_PLAQUETTE_FORCE, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_plaquette_force(F, (double*)ws, d_S, d_force, force_form, (cudaStream_t)stream));
}

int flue_meanlink(const flue_field* U, const void* G, int g_dtype, double* d_sum4, void* ws, size_t ws_bytes,
                  void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!G || !d_sum4) return fail(FLUE_ERR_ARG, "NULL pointer");
    if (g_dtype != FLUE_C128 && g_dtype != FLUE_C64) return fail(FLUE_ERR_DTYPE, "G must be c128 or c64");
    if ((rc = check_ws(FLUE_OP_MEANLINK, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_meanlink(F, G, g_dtype, (double*)ws, d_sum4, (cudaStream_t)stream));
}

int flue_gauge_transform(const flue_field* U, const void* G, int g_dtype, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!G) return fail(FLUE_ERR_ARG, "NULL gauge transformation");
    if (g_dtype != FLUE_C128 && g_dtype != FLUE_C64) return fail(FLUE_ERR_DTYPE, "G must be c128 or c64");
    if (((uintptr_t)G) % (g_dtype == FLUE_C64 ? 8 : 16)) return fail(FLUE_ERR_LAYOUT, "G pointer misaligned");
    return cuda_status(launch_gauge_transform(F, G, g_dtype, (cudaStream_t)stream));
}

int flue_gluon_propagator(const flue_field* U, double xi, int mu_start, double* d_D, void* ws, size_t ws_bytes,
                          void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (!d_D) return fail(FLUE_ERR_ARG, "NULL output");
    if (mu_start != 0 && mu_start != 1) return fail(FLUE_ERR_ARG, "mu_start must be 0 (all directions) or 1 (spatial)");
    if (!isfinite(xi)) return fail(FLUE_ERR_ARG, "xi must be finite");
    if ((rc = check_ws(FLUE_OP_GLUON_PROP, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_gluon_propagator(F, xi, mu_start, d_D, ws, ws_bytes, (cudaStream_t)stream));
}

int flue_wflow_step(const flue_field* U, double eps, void* ws, size_t ws_bytes, void* stream) {
    FieldRef F;
    int rc = check_field(U, &F);
    if (rc) return rc;
    if (F.prec == FLUE_R12) return fail(FLUE_ERR_DTYPE, "Wilson flow needs a C128 or C64 field");
    if (!(eps > 0.0) || !isfinite(eps)) return fail(FLUE_ERR_ARG, "eps must be positive");
    if ((rc = check_ws(FLUE_OP_WFLOW, F, ws_bytes, ws))) return rc;
    return cuda_status(launch_wflow_step((void*)F.links, F.g, F.prec, eps, ws, (cudaStream_t)stream));
}

}  // extern "C"

// ===========================================================================
// Host-buffer tier
// ===========================================================================
namespace {

struct DevCache {
    std::mutex mtx;
    bool init = false;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    void* field = nullptr;
    size_t field_bytes = 0;
    void* field2 = nullptr;
    size_t field2_bytes = 0;
    void* ws = nullptr;
    size_t ws_bytes = 0;
    void* out = nullptr;
    size_t out_bytes = 0;
    double* scal = nullptr;
    // large host<->device copies are split over several streams so that
    // more than one copy engine moves the bytes
    static constexpr int kCopyStreams = 4;
    int ncopy = 1;
    cudaStream_t cst[kCopyStreams] = {};
    cudaEvent_t cev[kCopyStreams + 1] = {};
    // T-slab pipeline of the host-buffer B^2 force (created on first use):
    // high-priority streams that stream slabs in (pack) and gradients out
    // beside the compute on `st` (and up to kPipeComp - 1 more compute
    // streams), a ring of kPipeComp + 1 buffer slots (packed slab + workspace)
    static constexpr int kPipeComp = 4, kPipeSlots = kPipeComp + 1;
    bool pipe_init = false;
    cudaStream_t s_in = nullptr, s_out = nullptr, s_cp[kPipeComp - 1] = {};
    cudaEvent_t ev_go = nullptr, ev_in[kPipeSlots] = {}, ev_cp[kPipeSlots] = {}, ev_out[kPipeSlots] = {},
                ev_end[kPipeComp - 1] = {};
    void* slot[kPipeSlots] = {};
    size_t slot_bytes[kPipeSlots] = {};
    // copy-engine transfers of pinned host buffers: chunks of time slices
    // copied in by 2-D DMA on s_dma into `stage` and out of the two chunk
    // buffers `ostage` on s_dout, one event per chunk
    static constexpr int kMaxChunks = 64;
    cudaStream_t s_dma = nullptr, s_dout = nullptr;
    cudaEvent_t ev_dma[kMaxChunks] = {}, ev_dout[kMaxChunks] = {};
    void* stage = nullptr;
    size_t stage_bytes = 0;
    void* ostage = nullptr;
    size_t ostage_bytes = 0;
};

// A device-usable address of host memory `p`, or NULL: pinned (page-locked,
// mapped) host memory, or -- when the GPU reads through the host's page
// tables, as GB300 with NVLink-C2C does -- any host memory.  Disabled with
// FLUE_ZERO_COPY=0.
static const void* device_view(const void* p) {
    const char* env = getenv("FLUE_ZERO_COPY");
    if (env && atoi(env) == 0) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
    int dev = 0, ats = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return ats ? p : nullptr;
}

// Pinned (page-locked) host memory that the host-buffer force moves by
// copy-engine copies: only when the environment variable `env_name`
// (FLUE_DMA_IN for the field, FLUE_DMA_OUT for the gradient) is set to a
// non-zero value; otherwise kernels read / write it.
static bool pinned_host(const void* p, const char* env_name) {
    const char* env = getenv(env_name);
    if (!env || atoi(env) == 0) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Copy `bytes` between host and device on the cache's stream, as one copy or
// split into chunks on the copy streams (ordered after everything queued on
// c->st before the call, and everything queued after it waits for all chunks).
static cudaError_t copy_async(DevCache* c, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    const size_t kMinSplit = (size_t)64 << 20;
    const char* env = getenv("FLUE_COPY_STREAMS");  // read per call: 1 = one copy
    const int n = env ? atoi(env) : DevCache::kCopyStreams;
    c->ncopy = n < 1 ? 1 : (n > DevCache::kCopyStreams ? DevCache::kCopyStreams : n);
    if (c->ncopy <= 1 || bytes < kMinSplit) return cudaMemcpyAsync(dst, src, bytes, kind, c->st);
    cudaError_t e = cudaEventRecord(c->cev[0], c->st);
    if (e != cudaSuccess) return e;
    const size_t chunk = ((bytes / c->ncopy) + 4095) & ~(size_t)4095;
    for (int k = 0; k < c->ncopy; ++k) {
        const size_t off = chunk * k;
        if (off >= bytes) break;
        const size_t n = (off + chunk > bytes) ? bytes - off : chunk;
        if ((e = cudaStreamWaitEvent(c->cst[k], c->cev[0], 0)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync((char*)dst + off, (const char*)src + off, n, kind, c->cst[k])) != cudaSuccess) return e;
        if ((e = cudaEventRecord(c->cev[k + 1], c->cst[k])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(c->st, c->cev[k + 1], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

std::mutex g_cache_mtx;
std::vector<DevCache*> g_caches;

int grow(void** p, size_t* have, size_t need) {
    if (*have >= need && *p) return FLUE_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(p, need < 256 ? 256 : need);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(FLUE_ERR_NOMEM, "device allocation failed in the host-buffer tier");
    }
    *have = need;
    return FLUE_OK;
}

DevCache* cache_for_current(int* rc) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *rc = cuda_status(e);
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_cache_mtx);
    if ((int)g_caches.size() <= dev) g_caches.resize(dev + 1, nullptr);
    if (!g_caches[dev]) g_caches[dev] = new DevCache();
    DevCache* c = g_caches[dev];
    if (!c->init) {
        if ((e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreate(&c->e0)) != cudaSuccess || (e = cudaEventCreate(&c->e1)) != cudaSuccess ||
            (e = cudaMalloc((void**)&c->scal, 64 * sizeof(double))) != cudaSuccess) {
            *rc = cuda_status(e);
            return nullptr;
        }
        for (int k = 0; k < DevCache::kCopyStreams; ++k)
            if ((e = cudaStreamCreateWithFlags(&c->cst[k], cudaStreamNonBlocking)) != cudaSuccess) {
                *rc = cuda_status(e);
                return nullptr;
            }
        for (int k = 0; k <= DevCache::kCopyStreams; ++k)
            if ((e = cudaEventCreateWithFlags(&c->cev[k], cudaEventDisableTiming)) != cudaSuccess) {
                *rc = cuda_status(e);
                return nullptr;
            }
        c->init = true;
    }
    *rc = FLUE_OK;
    return c;
}

// Upload a host complex128 field (Fortran order) into the cache's field
// buffer; the reference layout IS the FLUE_C128 device layout.
int upload_c128(DevCache* c, const double* data, int nt, int nx, int ny, int nz, flue_field* U) {
    if (!data) return fail(FLUE_ERR_ARG, "NULL data");
    if (!dims_ok(nt, nx, ny, nz)) return fail(FLUE_ERR_SHAPE, "bad lattice extents");
    const size_t bytes = (size_t)flue_field_bytes(nt, nx, ny, nz, FLUE_C128);
    int rc = grow(&c->field, &c->field_bytes, bytes);
    if (rc) return rc;
    cudaError_t e = copy_async(c, c->field, data, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e);
    U->links = c->field;
    U->nt = nt;
    U->nx = nx;
    U->ny = ny;
    U->nz = nz;
    U->prec = FLUE_C128;
    return FLUE_OK;
}

int ensure_ws(DevCache* c, int op, const flue_field& U) {
    const size_t need = flue_workspace_bytes(op, U.nt, U.nx, U.ny, U.nz, U.prec);
    return grow(&c->ws, &c->ws_bytes, need);
}

int fetch(DevCache* c, void* host, const void* dev, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->st);
    if (e != cudaSuccess) return cuda_status(e);
    return cuda_status(cudaStreamSynchronize(c->st));
}

double elapsed_s(DevCache* c) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->e0, c->e1);
    return (double)ms * 1e-3;
}

// Host-buffer B^2 and gradient, pipelined over time slabs.  B^2 uses only
// spatial planes, so time slices are independent: slab k (nts time slices)
// is packed from host memory on s_in, computed (lines, forward, line
// cotangents) on compute stream k % ncomp, and its link cotangents are
// written into the host gradient on s_out, while later slabs are packed and
// earlier ones written out.
// The two I/O streams have the highest priority and capped grids, so they
// take a few SMs and the host link (NVLink-C2C) while compute keeps the rest.
// Per-slab B^2 partials are added on the host in slab order (deterministic).
int pipe_setup(DevCache* c) {
    if (c->pipe_init) return FLUE_OK;
    int lo = 0, hi = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->s_in, cudaStreamNonBlocking, hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->s_out, cudaStreamNonBlocking, hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_go, cudaEventDisableTiming);
    for (int j = 0; j < DevCache::kPipeSlots && e == cudaSuccess; ++j) {
        e = cudaEventCreateWithFlags(&c->ev_in[j], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_cp[j], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out[j], cudaEventDisableTiming);
    }
    for (int i = 0; i < DevCache::kPipeComp - 1 && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&c->s_cp[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_end[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->s_dma, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->s_dout, cudaStreamNonBlocking);
    for (int q = 0; q < DevCache::kMaxChunks && e == cudaSuccess; ++q) {
        e = cudaEventCreateWithFlags(&c->ev_dma[q], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_dout[q], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return cuda_status(e);
    c->pipe_init = true;
    return FLUE_OK;
}

int env_int(const char* name, int dflt) {
    const char* v = getenv(name);
    return v ? atoi(v) : dflt;
}

// Number of time slabs for the pipelined host-buffer B^2 force: FLUE_SLABS,
// else slabs of at least 8 time slices and 2^17 sites, at most 16 slabs;
// 1 = no pipelining.
int pipe_slabs(int NT, int64_t V) {
    int s = env_int("FLUE_SLABS", 0);
    if (s <= 0) {
        // slabs of a power-of-two number of slices, >= 4 and >= 2^17 sites,
        // at most 16 of them (measured at 64x32^3: 16 slabs of 4 slices 11.47 ms
        // per call, 8 of 8 slices 11.70 ms)
        const int64_t v3 = V / NT;
        int nts = 4;
        while (nts < NT && ((int64_t)nts * v3 < ((int64_t)1 << 17) || (NT + nts - 1) / nts > 16)) nts *= 2;
        s = (NT + nts - 1) / nts;
    }
    if (s > NT) s = NT;
    if (s > 32) s = 32;  // per-slab partials live in the 64-double scalar buffer
    return s < 1 ? 1 : s;
}

// Host memory that the CPU may write (pinned or pageable; not device or
// managed memory).
static bool cpu_writable(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeUnregistered;
}

// Zero-fills the listed byte ranges of host memory on up to 8 threads,
// started at construction and joined at destruction (a share whose thread
// cannot be started is zeroed on the calling thread).
struct HostZeroFill {
    std::vector<std::thread> th;
    HostZeroFill(const std::vector<std::pair<char*, size_t>>& ranges) {
        size_t total = 0;
        for (auto& r : ranges) total += r.second;
        unsigned hw = std::thread::hardware_concurrency();
        const size_t nt = hw == 0 ? 4 : (hw < 8 ? hw : 8);
        const size_t per = (total + nt - 1) / nt;
        // share k: bytes [k * per, (k + 1) * per) of the ranges laid end to end
        auto share = [ranges, per](size_t k) {
            size_t lo = k * per, hi = lo + per, at = 0;
            for (auto& r : ranges) {
                const size_t a = lo > at ? lo : at, b = hi < at + r.second ? hi : at + r.second;
                if (a < b) memset(r.first + (a - at), 0, b - a);
                at += r.second;
            }
        };
        for (size_t k = 0; k < nt && per; ++k) {
            try {
                th.emplace_back(share, k);
            } catch (...) {
                share(k);
            }
        }
    }
    ~HostZeroFill() {
        for (auto& t : th) t.join();
    }
};

int magnetic_force_pipelined(DevCache* c, const void* d_in, const void* h_in, void* h_grad, int data_dtype, int NT,
                             int NX, int NY, int NZ, int prec, int form, double* B, void* d_grad, int nslab,
                             void* cpu_grad) {
    int rc = pipe_setup(c);
    if (rc) return rc;
    const int64_t V = (int64_t)NT * NX * NY * NZ;
    const int64_t V3 = V / NT;
    const int64_t st[7] = {1, NT, (int64_t)NT * NX, (int64_t)NT * NX * NY, V, 4 * V, 12 * V};
    const int nts = (NT + nslab - 1) / nslab;
    nslab = (NT + nts - 1) / nts;
    const size_t esz = data_dtype == FLUE_C128 ? 16 : 8;
    // Copy-engine transfers of pinned host buffers (h_in: the field, h_grad:
    // the gradient; opt-in, FLUE_DMA_IN / FLUE_DMA_OUT = 1).  Kernels that
    // read or write host memory hold SMs while they wait on the host link and
    // share one budget of it (measured on GB300 at 64x32^3 complex128:
    // reading the field's stored rows 3.8 ms, writing the gradient 6.2 ms,
    // both at once 10.1 ms; in the pipeline the gradient writes, 0.63 ms per
    // slab, set the pace), while the copy engines use no SMs and move both
    // directions at once (1.2 GB each way in 7.1 ms).  A 2-D copy moves rows
    // of CH time slices of every (column, direction, matrix element) between
    // the host array and a chunk buffer: 256-byte rows ran at 185 GB/s,
    // 128-byte at 107, 64-byte at 56.  The first chunk's slabs read the field
    // with kernels, and the copies of the other chunks start after them
    // (copies that start at once take the host link from those reads and
    // delay every compute); the last FLUE_OUT_TAIL slabs write their gradient
    // with kernels.  Reconstruct-12 stages the first two matrix rows only.
    // Measured per call at 64x32^3, 16 slabs of 4 slices, r12, 60 calls
    // (kernel reads and writes -> copies): complex128 median 11.24 -> 10.39 ms
    // with 16-slice chunks and no kernel-written tail (8-slice chunks 12.5,
    // 32-slice 12.1-13.2), complex64 9.43 -> 9.20 ms with a tail of 2; but
    // one call in 15-60 has a single copy stall for 6-27 ms (with or without
    // other transfers beside it, whole or split into pieces of 16384 or 4096
    // rows), against a spread of 10.9-11.6 ms with kernel transfers -- so the
    // copies stay opt-in.
    const int ch_env = env_int("FLUE_DMA_CHUNK", 16);  // slices per chunk, rounded up to whole slabs
    int CH = nts * (int)(((ch_env > 0 ? ch_env : 16) + nts - 1) / nts);
    if (CH > NT) CH = NT;
    const int nchunk = (NT + CH - 1) / CH;
    if (nchunk < 2 || nchunk > DevCache::kMaxChunks) h_in = h_grad = nullptr;
    if (!d_grad) h_grad = nullptr;
    // Slab schedule.  Each slab reads, per site column, a run of n time
    // slices (n * esz bytes) from host memory; runs that straddle 64-byte
    // boundaries cost extra transfers over the host link (measured: a numpy
    // array, 16 bytes past a page boundary, 14.5 ms per call against 11.8 ms
    // aligned).  A run of A = min(64, n * esz) bytes (a power of two) that
    // starts on an A-byte boundary stays inside one 64-byte block, so when
    // the field's address is off an A-byte boundary by a whole number of
    // elements, a short first slab shifts the grid so that every later
    // slab's runs start on one (not with copy-engine chunks, whose slabs
    // start on multiples of the slab length).
    size_t A = 64;
    while (A > esz && A > (size_t)nts * esz) A >>= 1;
    int t0s[34], ns[34];
    int nsl = 0;
    {
        const size_t off = (size_t)((uintptr_t)d_in % A);
        int first = (off && off % esz == 0) ? (int)((A - off) / esz) : 0;
        if (first >= nts || first >= NT || nslab >= 33 || h_in || h_grad) first = 0;
        int t = 0;
        if (first) t0s[nsl] = 0, ns[nsl++] = first, t = first;
        while (t < NT) {
            const int n = NT - t < nts ? NT - t : nts;
            t0s[nsl] = t, ns[nsl++] = n, t += n;
        }
    }
    nslab = nsl;
    // input staging: chunk q >= 1, plane (a, b) with a < R, direction mu,
    // column, slice in the chunk
    const int R = prec == FLUE_R12 ? 2 : 3;
    const int64_t P = 4 * V3 * (int64_t)CH;  // elements per plane and chunk
    if (h_in && (rc = grow(&c->stage, &c->stage_bytes, (size_t)(nchunk - 1) * R * 3 * P * esz))) return rc;
    const int64_t sst[7] = {1, CH, (int64_t)CH * NX, (int64_t)CH * NX * NY, (int64_t)CH * V3, P, (int64_t)R * P};
    // output staging: two chunk buffers holding a gradient of time extent CH
    // (slices [0, Tdma) leave by copies, the tail by kernel writes)
    int ztail = env_int("FLUE_OUT_TAIL", esz == 16 ? 0 : 2);
    ztail = ztail < 0 ? 0 : ztail;
    const int Tdma = !h_grad ? 0 : (ztail == 0 ? NT : (nslab > ztail ? t0s[nslab - ztail] : 0));
    const size_t Bo = (size_t)(9 * P) * esz;
    if (Tdma && (rc = grow(&c->ostage, &c->ostage_bytes, 2 * Bo))) return rc;
    const PlaneSet ps = b2_planes();
    const Geom g0 = make_geom(nts, NX, NY, NZ);
    const size_t fbytes = ((size_t)flue_field_bytes(nts, NX, NY, NZ, prec) + 255) & ~(size_t)255;
    const size_t wbytes = energy_ws_bytes(g0, prec, ps, d_grad != nullptr);
    // compute streams (FLUE_PIPE_STREAMS, default 3): slab k computes on
    // stream k % ncomp, so the compute of neighbouring slabs overlaps too
    // (measured at 64x32^3, 8 slabs: 12.5 ms on 1 stream, 11.9 on 2, 11.8 on 3;
    // 16 slabs: 11.7 on 2, 11.4 on 3 and on 4)
    int ncomp = env_int("FLUE_PIPE_STREAMS", 3);
    ncomp = ncomp < 1 ? 1 : (ncomp > DevCache::kPipeComp ? DevCache::kPipeComp : ncomp);
    const int nslot = ncomp + 1;
    for (int j = 0; j < nslot; ++j)
        if ((rc = grow(&c->slot[j], &c->slot_bytes[j], fbytes + wbytes))) return rc;
    // grid caps of the I/O kernels (FLUE_IN_BLOCKS, FLUE_OUT_BLOCKS): measured
    // on GB300 at 64x32^3, 8 slabs, one compute stream: 32 pack blocks of 256
    // threads and 16 x 4 output blocks of 128 give 12.4 ms per call against
    // 16.9 ms unpipelined; uncapped I/O grids take every SM and serialise with
    // compute (16.9 ms), 8 / 4 starve the host link (22 ms)
    // The first pack and the last write-out have no compute beside them and
    // run on the whole GPU (8 slabs: 11.95 -> 11.79 ms per call).
    const unsigned in_blocks = (unsigned)env_int("FLUE_IN_BLOCKS", 32);
    // (with the time direction off the link, same box, median per call: a
    // complex128 field 9.68 ms with 16 x 4 output blocks, 9.53 with 12 x 4;
    // complex64 9.09 with 16, 9.12 with 12)
    const unsigned out_blocks = (unsigned)env_int("FLUE_OUT_BLOCKS", esz == 16 ? 12 : 16);
    // B^2 has no plane with the time direction: its links are not packed
    // (pmu0 = 1) and its gradient is zero.  With the gradient in host memory
    // the CPU writes those zeros while the GPU computes, so that only the
    // spatial directions cross the host link, 3/4 of the bytes each way
    // (FLUE_HOST_ZERO=0: the GPU writes them; with copy-engine output too).
    // Measured at 64x32^3 r12, same box, median per call: complex128 11.25 ms
    // -> 10.94 (spatial pack) -> 9.66 (and host zeros); complex64 9.39 ->
    // 9.16 ms.
    const int pmu0 = 1;
    std::unique_ptr<HostZeroFill> zfill;
    if (cpu_grad && d_grad && !Tdma && env_int("FLUE_HOST_ZERO", 1)) {
        std::vector<std::pair<char*, size_t>> r;
        for (int ab = 0; ab < 9; ++ab) r.push_back({(char*)cpu_grad + (size_t)(4 * V * ab) * esz, (size_t)V * esz});
        zfill.reset(new HostZeroFill(r));
    }
    cudaError_t e = cudaEventRecord(c->ev_go, c->st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->s_in, c->ev_go, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->s_out, c->ev_go, 0);
    if (e == cudaSuccess && Tdma) e = cudaStreamWaitEvent(c->s_dout, c->ev_go, 0);
    for (int i = 1; i < ncomp && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(c->s_cp[i - 1], c->ev_go, 0);
    // the slab after whose read the field's copies start (FLUE_DMA_AFTER,
    // default the first chunk's last slab)
    int kdma = env_int("FLUE_DMA_AFTER", CH / nts - 1);
    kdma = kdma < 0 ? 0 : (kdma > CH / nts - 1 ? CH / nts - 1 : kdma);
    int last_dout = -1;
    for (int k = 0; k < nslab && e == cudaSuccess; ++k) {
        const int j = k % nslot, t0 = t0s[k], n = ns[k];
        cudaStream_t cs = (k % ncomp) == 0 ? c->st : c->s_cp[k % ncomp - 1];
        const Geom g = make_geom(n, NX, NY, NZ);
        char* buf = (char*)c->slot[j];
        const FieldRef U{buf, g, prec};
        // pack slab k once the compute of slab k - nslot has read this slot
        if (k >= nslot && (e = cudaStreamWaitEvent(c->s_in, c->ev_cp[j], 0)) != cudaSuccess) break;
        if (h_in && t0 >= CH) {
            // from the staged chunk holding slices [t0, t0 + n)
            const int q = t0 / CH;
            if ((e = cudaStreamWaitEvent(c->s_in, c->ev_dma[q], 0)) != cudaSuccess) break;
            const char* src = (const char*)c->stage + (size_t)((int64_t)(q - 1) * R * 3 * P + (t0 - q * CH)) * esz;
            if ((e = launch_pack(src, data_dtype, sst, g, buf, prec, 0, c->s_in, in_blocks, pmu0)) != cudaSuccess) break;
        } else if ((e = launch_pack((const char*)d_in + (size_t)t0 * esz, data_dtype, st, g, buf, prec, 0, c->s_in,
                                    k == 0 ? 0u : in_blocks, pmu0)) != cudaSuccess) {
            break;
        }
        if ((e = cudaEventRecord(c->ev_in[j], c->s_in)) != cudaSuccess) break;
        if (h_in && k == kdma) {
            // chunks 1.. of the field, back to back on the copy stream once
            // the first slabs have been read (before, the copies take the
            // host link from the reads the first computes wait for)
            if ((e = cudaStreamWaitEvent(c->s_dma, c->ev_in[j], 0)) != cudaSuccess) break;
            for (int q = 1; q < nchunk && e == cudaSuccess; ++q) {
                const int tq = q * CH, nq = NT - tq < CH ? NT - tq : CH;
                for (int b = 0; b < 3 && e == cudaSuccess; ++b)
                    for (int a = 0; a < R && e == cudaSuccess; ++a) {
                        const char* hs = (const char*)h_in + (size_t)(4 * V * (a + 3 * b) + tq) * esz;
                        char* dst = (char*)c->stage + (size_t)((q - 1) * R * 3 * P + (a + (int64_t)R * b) * P) * esz;
                        e = cudaMemcpy2DAsync(dst + (size_t)V3 * CH * esz, (size_t)CH * esz, hs + (size_t)V * esz,
                                              (size_t)NT * esz, (size_t)nq * esz, (size_t)(3 * V3),
                                              cudaMemcpyHostToDevice, c->s_dma);
                    }
                if (e == cudaSuccess) e = cudaEventRecord(c->ev_dma[q], c->s_dma);
            }
            if (e != cudaSuccess) break;
        }
        // compute slab k once it is packed and the output of slab k - nslot
        // has left this slot's workspace
        if ((e = cudaStreamWaitEvent(cs, c->ev_in[j], 0)) != cudaSuccess) break;
        if (k >= nslot && d_grad && (e = cudaStreamWaitEvent(cs, c->ev_out[j], 0)) != cudaSuccess) break;
        if ((e = launch_energy_slab_fwd(U, 0, n, ps, V, c->scal + k, d_grad != nullptr, buf + fbytes, wbytes, cs)) !=
            cudaSuccess)
            break;
        if ((e = cudaEventRecord(c->ev_cp[j], cs)) != cudaSuccess) break;
        if (!d_grad) continue;
        if (t0 < Tdma) {
            // gradient into the chunk buffer on the compute stream, once the
            // copy of the chunk two before has left it; the chunk's copy
            // follows its last slab
            const int q = t0 / CH, tend = (q + 1) * CH < Tdma ? (q + 1) * CH : Tdma;
            if (q >= 2 && (e = cudaStreamWaitEvent(cs, c->ev_dout[q - 2], 0)) != cudaSuccess) break;
            char* ob = (char*)c->ostage + (size_t)(q % 2) * Bo;
            if ((e = launch_energy_slab_out(U, ps, V, CH, t0 - q * CH, ob, form, buf + fbytes, wbytes, 0, cs,
                                            data_dtype)) != cudaSuccess)
                break;
            if ((e = cudaEventRecord(c->ev_out[j], cs)) != cudaSuccess) break;
            if ((e = cudaStreamWaitEvent(c->s_dout, c->ev_out[j], 0)) != cudaSuccess) break;
            if (t0 + n == tend) {
                e = cudaMemcpy2DAsync((char*)h_grad + (size_t)q * CH * esz, (size_t)NT * esz, ob, (size_t)CH * esz,
                                      (size_t)(tend - q * CH) * esz, (size_t)(36 * V3), cudaMemcpyDeviceToHost,
                                      c->s_dout);
                if (e == cudaSuccess) e = cudaEventRecord(c->ev_dout[q], c->s_dout);
                if (e != cudaSuccess) break;
                last_dout = q;
            }
            continue;
        }
        if ((e = cudaStreamWaitEvent(c->s_out, c->ev_cp[j], 0)) != cudaSuccess) break;
        const unsigned ob = k == nslab - 1 ? 0u : out_blocks;
        if ((e = launch_energy_slab_out(U, ps, V, NT, t0, d_grad, form, buf + fbytes, wbytes, ob, c->s_out,
                                        data_dtype, zfill != nullptr)) != cudaSuccess)
            break;
        if ((e = cudaEventRecord(c->ev_out[j], c->s_out)) != cudaSuccess) break;
    }
    // every stream joins st before the partials are read (also after an error)
    for (int i = 1; i < ncomp; ++i) {
        cudaError_t r = cudaEventRecord(c->ev_end[i - 1], c->s_cp[i - 1]);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(c->st, c->ev_end[i - 1], 0);
        if (e == cudaSuccess) e = r;
    }
    if (e == cudaSuccess && d_grad) e = cudaStreamWaitEvent(c->st, c->ev_out[(nslab - 1) % nslot], 0);
    if (e == cudaSuccess && last_dout >= 0) e = cudaStreamWaitEvent(c->st, c->ev_dout[last_dout], 0);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(c->s_dma);
        cudaStreamSynchronize(c->s_in);
        cudaStreamSynchronize(c->s_out);
        cudaStreamSynchronize(c->s_dout);
        for (int i = 1; i < ncomp; ++i) cudaStreamSynchronize(c->s_cp[i - 1]);
        cudaStreamSynchronize(c->st);
        return cuda_status(e);
    }
    double part[34];
    if ((rc = fetch(c, part, c->scal, sizeof(double) * nslab))) return rc;
    double b = 0.0;
    for (int k = 0; k < nslab; ++k) b += part[k];
    *B = b;
    return FLUE_OK;
}

}  // namespace

#define HOST_PROLOGUE()                        \
    int rc = FLUE_OK;                          \
    DevCache* c = cache_for_current(&rc);      \
    if (!c) return rc;                         \
    std::lock_guard<std::mutex> lk(c->mtx)

extern "C" {

static int plaq_host(const double* data, int NT, int NX, int NY, int NZ, int muStart, int muEnd, int nuEnd,
                     double* sumTrP, int* nP, double* time) {
    if (!sumTrP || !nP || !time) return fail(FLUE_ERR_ARG, "NULL output");
    HOST_PROLOGUE();
    flue_field U;
    if ((rc = upload_c128(c, data, NT, NX, NY, NZ, &U))) return rc;
    if ((rc = ensure_ws(c, FLUE_OP_PLAQUETTE, U))) return rc;
    cudaEventRecord(c->e0, c->st);
    if ((rc = flue_plaquette(&U, muStart, muEnd, nuEnd, c->scal, c->ws, c->ws_bytes, c->st))) return rc;
    cudaEventRecord(c->e1, c->st);
    double s = 0.0;
    if ((rc = fetch(c, &s, c->scal, sizeof(double)))) return rc;
    int np = 0;
    for (int mu = muStart; mu <= muEnd; ++mu)
        for (int nu = mu + 1; nu <= nuEnd; ++nu) np++;
    *sumTrP = s;
    *nP = (int)((int64_t)np * NT * NX * NY * NZ);
    *time = elapsed_s(c);
    return FLUE_OK;
}

int flue_plaquette_c(const double* data, int NT, int NX, int NY, int NZ, int muStart, int muEnd, int nuEnd,
                     double* sumTrP, int* nP, double* time) {
    return plaq_host(data, NT, NX, NY, NZ, muStart, muEnd, nuEnd, sumTrP, nP, time);
}

int flue_genplaquette_c(const double* data, int NT, int NX, int NY, int NZ, int muStart, int muEnd, int nuEnd,
                        double* sumTrP, int* nP, double* time) {
    return plaq_host(data, NT, NX, NY, NZ, muStart, muEnd, nuEnd, sumTrP, nP, time);
}

int flue_polyakov_c(const double* data, int NT, int NX, int NY, int NZ, double* sumTrP, int* nP, double* time) {
    if (!sumTrP || !nP || !time) return fail(FLUE_ERR_ARG, "NULL output");
    HOST_PROLOGUE();
    flue_field U;
    if ((rc = upload_c128(c, data, NT, NX, NY, NZ, &U))) return rc;
    if ((rc = ensure_ws(c, FLUE_OP_POLYAKOV, U))) return rc;
    cudaEventRecord(c->e0, c->st);
    if ((rc = flue_polyakov(&U, c->scal, c->ws, c->ws_bytes, c->st))) return rc;
    cudaEventRecord(c->e1, c->st);
    double s[2];
    if ((rc = fetch(c, s, c->scal, 2 * sizeof(double)))) return rc;
    *sumTrP = s[0];
    *nP = NX * NY * NZ;
    *time = elapsed_s(c);
    return FLUE_OK;
}

int flue_genericpath_c(const double* data, int NT, int NX, int NY, int NZ, const int* coordBase, const int* path,
                       int npath, double* U_xd) {
    if (!U_xd || !coordBase) return fail(FLUE_ERR_ARG, "NULL pointer");
    HOST_PROLOGUE();
    flue_field U;
    if ((rc = upload_c128(c, data, NT, NX, NY, NZ, &U))) return rc;
    if ((rc = grow(&c->out, &c->out_bytes, 9 * 16))) return rc;
    if ((rc = flue_genericpath(&U, coordBase, path, npath, c->out, c->st))) return rc;
    return fetch(c, U_xd, c->out, 9 * 16);
}

static int wloop_host(const double* data, int NT, int NX, int NY, int NZ, int tau, int mu, int nu, int nMu, int nNu,
                      double* loopVal) {
    if (!loopVal) return fail(FLUE_ERR_ARG, "NULL output");
    HOST_PROLOGUE();
    flue_field U;
    if ((rc = upload_c128(c, data, NT, NX, NY, NZ, &U))) return rc;
    if ((rc = ensure_ws(c, FLUE_OP_WMUNU, U))) return rc;
    if ((rc = flue_wmunu(&U, tau, mu, nu, nMu, nNu, c->scal, c->ws, c->ws_bytes, c->st))) return rc;
    return fetch(c, loopVal, c->scal, sizeof(double));
}

int flue_wmunu_c(const double* data, int NT, int NX, int NY, int NZ, int mu, int nu, int nMu, int nNu, double* loopVal) {
    return wloop_host(data, NT, NX, NY, NZ, 0, mu, nu, nMu, nNu, loopVal);
}

int flue_wmunutau_c(const double* data, int NT, int NX, int NY, int NZ, int tau, int mu, int nu, int nMu, int nNu,
                    double* loopVal) {
    if (tau < 1) return fail(FLUE_ERR_ARG, "tau out of 1..NT");
    return wloop_host(data, NT, NX, NY, NZ, tau, mu, nu, nMu, nNu, loopVal);
}

static int fmunu_host(const double* data, int NT, int NX, int NY, int NZ, int kind, int mu, int nu, double* U_xd) {
    if (!U_xd) return fail(FLUE_ERR_ARG, "NULL output");
    HOST_PROLOGUE();
    flue_field U;
    if ((rc = upload_c128(c, data, NT, NX, NY, NZ, &U))) return rc;
    if ((rc = ensure_ws(c, FLUE_OP_FMUNU, U))) return rc;
    const size_t ob = (size_t)NT * NX * NY * NZ * 9 * 16;
    if ((rc = grow(&c->out, &c->out_bytes, ob))) return rc;
    if ((rc = flue_fmunu(&U, kind, mu, nu, c->out, c->ws, c->ws_bytes, c->st))) return rc;
    return fetch(c, U_xd, c->out, ob);
}

int flue_cloverloopmunucoord_c(const double* data, int NT, int NX, int NY, int NZ, int mu, int nu, double* U_xd) {
    return fmunu_host(data, NT, NX, NY, NZ, FLUE_FMUNU_CLOVER, mu, nu, U_xd);
}

int flue_loop5munucoord_c(const double* data, int NT, int NX, int NY, int NZ, int mu, int nu, double* U_xd) {
    return fmunu_host(data, NT, NX, NY, NZ, FLUE_FMUNU_LOOP5, mu, nu, U_xd);
}

int flue_magnetic_c(const double* data, int NT, int NX, int NY, int NZ, double* B) {
    if (!B) return fail(FLUE_ERR_ARG, "NULL output");
    HOST_PROLOGUE();
    flue_field U;
    if ((rc = upload_c128(c, data, NT, NX, NY, NZ, &U))) return rc;
    if ((rc = ensure_ws(c, FLUE_OP_MAGNETIC, U))) return rc;
    if ((rc = flue_magnetic(&U, c->scal, c->ws, c->ws_bytes, c->st))) return rc;
    return fetch(c, B, c->scal, sizeof(double));
}

int flue_multiplymatmat_c(double* MM, const double* left, const double* right) {
    if (!MM || !left || !right) return fail(FLUE_ERR_ARG, "NULL pointer");
    HOST_PROLOGUE();
    if ((rc = grow(&c->out, &c->out_bytes, 3 * 9 * 16))) return rc;
    char* o = (char*)c->out;
    cudaError_t e = cudaMemcpyAsync(o, left, 9 * 16, cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(o + 9 * 16, right, 9 * 16, cudaMemcpyHostToDevice, c->st);
    if (e != cudaSuccess) return cuda_status(e);
    if ((rc = flue_multiplymatmat_batch(o, o + 9 * 16, o + 18 * 16, 1, FLUE_C128, 0, c->st))) return rc;
    return fetch(c, MM, o + 18 * 16, 9 * 16);
}

int flue_fixsu3matrix_c(double* U_x) {
    if (!U_x) return fail(FLUE_ERR_ARG, "NULL pointer");
    HOST_PROLOGUE();
    if ((rc = grow(&c->out, &c->out_bytes, 2 * 9 * 16))) return rc;
    char* o = (char*)c->out;
    cudaError_t e = cudaMemcpyAsync(o, U_x, 9 * 16, cudaMemcpyHostToDevice, c->st);
    if (e != cudaSuccess) return cuda_status(e);
    // one 3x3 matrix as a 1-site field with a single direction: strides of
    // (t,x,y,z,mu,a,b) = (0,0,0,0,0,1,3)
    const int64_t st[7] = {0, 0, 0, 0, 0, 1, 3};
    // pack into a 1x1x1x1 C128 field (4 directions, all the same matrix)
    if ((rc = grow(&c->field2, &c->field2_bytes, 36 * 16))) return rc;
    if ((rc = flue_pack_field(o, FLUE_C128, st, 1, 1, 1, 1, c->field2, FLUE_C128, 1, c->st))) return rc;
    // direction 0 of site 0: element (a,b) at 4*(a+3b)
    double tmp[36 * 2];
    if ((rc = fetch(c, tmp, c->field2, 36 * 16))) return rc;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            U_x[2 * (a + 3 * b)] = tmp[2 * 4 * (a + 3 * b)];
            U_x[2 * (a + 3 * b) + 1] = tmp[2 * 4 * (a + 3 * b) + 1];
        }
    return FLUE_OK;
}

int flue_uzerobar_c(const double* data, int NT, int NX, int NY, int NZ, const double* G, double* u0) {
    if (!u0) return fail(FLUE_ERR_ARG, "NULL output");
    HOST_PROLOGUE();
    flue_field U;
    if ((rc = upload_c128(c, data, NT, NX, NY, NZ, &U))) return rc;
    if ((rc = ensure_ws(c, FLUE_OP_MEANLINK, U))) return rc;
    const size_t need2 = flue_workspace_bytes(FLUE_OP_PLAQUETTE, NT, NX, NY, NZ, FLUE_C128);
    if (need2 > c->ws_bytes && (rc = grow(&c->ws, &c->ws_bytes, need2))) return rc;
    const int ranges[3][3] = {{1, 4, 4}, {2, 4, 4}, {1, 1, 4}};
    for (int k = 0; k < 3; ++k)
        if ((rc = flue_plaquette(&U, ranges[k][0], ranges[k][1], ranges[k][2], c->scal + k, c->ws, c->ws_bytes, c->st)))
            return rc;
    if (G) {
        const size_t gb = (size_t)NT * NX * NY * NZ * 9 * 16;
        if ((rc = grow(&c->out, &c->out_bytes, gb))) return rc;
        cudaError_t e = cudaMemcpyAsync(c->out, G, gb, cudaMemcpyHostToDevice, c->st);
        if (e != cudaSuccess) return cuda_status(e);
        if ((rc = flue_meanlink(&U, c->out, FLUE_C128, c->scal + 3, c->ws, c->ws_bytes, c->st))) return rc;
    }
    double s[7];
    if ((rc = fetch(c, s, c->scal, 7 * sizeof(double)))) return rc;
    const double V = (double)NT * NX * NY * NZ;
    const double p_all = s[0] / (6.0 * V) / 3.0, p_s = s[1] / (3.0 * V) / 3.0, p_t = s[2] / (3.0 * V) / 3.0;
    u0[0] = pow(p_all, 0.25);
    u0[1] = pow(p_s, 0.25);
    u0[2] = sqrt(p_t) / u0[1];
    if (G) {
        u0[3] = (s[3] + s[4] + s[5] + s[6]) / (4.0 * V) / 3.0;
        u0[4] = (s[4] + s[5] + s[6]) / (3.0 * V) / 3.0;
        u0[5] = s[3] / V / 3.0;
    } else {
        u0[3] = u0[4] = u0[5] = NAN;
    }
    return FLUE_OK;
}

int flue_scalargluonprop_c(int NS, int NT, const void* U, double xi, double* D) {
    if (!U || !D) return fail(FLUE_ERR_ARG, "NULL pointer");
    HOST_PROLOGUE();
    flue_field F;
    if ((rc = upload_c128(c, (const double*)U, NT, NS, NS, NS, &F))) return rc;
    if ((rc = ensure_ws(c, FLUE_OP_GLUON_PROP, F))) return rc;
    const size_t db = (size_t)NT * NS * NS * NS * sizeof(double);
    if ((rc = grow(&c->out, &c->out_bytes, db))) return rc;
    if ((rc = flue_gluon_propagator(&F, xi, 0, (double*)c->out, c->ws, c->ws_bytes, c->st))) return rc;
    return fetch(c, D, c->out, db);
}

int flue_magnetic_force_c(const void* data, int data_dtype, int NT, int NX, int NY, int NZ, int prec, int force_form,
                          double* B, void* grad) {
    if (!data || !B) return fail(FLUE_ERR_ARG, "NULL pointer");
    if (data_dtype != FLUE_C128 && data_dtype != FLUE_C64) return fail(FLUE_ERR_DTYPE, "data must be c128 or c64");
    if (!prec_ok(prec)) return fail(FLUE_ERR_DTYPE, "bad precision");
    if (data_dtype == FLUE_C64 && prec == FLUE_C128)
        return fail(FLUE_ERR_DTYPE, "c64 data is computed in FLUE_C64 or FLUE_R12");
    if (!dims_ok(NT, NX, NY, NZ)) return fail(FLUE_ERR_SHAPE, "bad lattice extents");
    HOST_PROLOGUE();
    const size_t in_bytes = (size_t)flue_field_bytes(NT, NX, NY, NZ, data_dtype);
    const int64_t V = (int64_t)NT * NX * NY * NZ;
    const int64_t st[7] = {1, NT, (int64_t)NT * NX, (int64_t)NT * NX * NY, V, 4 * V, 12 * V};
    // Zero copy: when the GPU can address the caller's host buffers (pinned
    // memory, or any memory on a system whose GPU walks the host page tables,
    // as over NVLink-C2C), the re-layout kernel reads the field straight from
    // host memory and the gradient kernel writes straight into it -- no
    // staging copies.  Otherwise the field is copied in and the gradient out.
    const void* d_in = device_view(data);
    void* d_grad = grad ? const_cast<void*>(device_view(grad)) : nullptr;
    if (d_in && (!grad || d_grad)) {
        const int nslab = pipe_slabs(NT, V);
        if (nslab > 1)
            return magnetic_force_pipelined(c, d_in, pinned_host(data, "FLUE_DMA_IN") ? data : nullptr,
                                            grad && pinned_host(grad, "FLUE_DMA_OUT") ? grad : nullptr, data_dtype,
                                            NT, NX, NY, NZ, prec, force_form, B, d_grad, nslab,
                                            grad && cpu_writable(grad) ? grad : nullptr);
    }
    flue_field U = {nullptr, NT, NX, NY, NZ, prec};
    // a complex128 field computed in FP32 (c128 data, prec C64 / R12) gets
    // its FP32 gradient widened back to complex128 before it leaves the GPU
    const bool widen = data_dtype == FLUE_C128 && prec != FLUE_C128;
    if (d_in) {
        const size_t fb = (size_t)flue_field_bytes(NT, NX, NY, NZ, prec);
        if ((rc = grow(&c->field2, &c->field2_bytes, fb))) return rc;
        if ((rc = flue_pack_field(d_in, data_dtype, st, NT, NX, NY, NZ, c->field2, prec, 0, c->st))) return rc;
        U.links = c->field2;
    } else {
        if ((rc = grow(&c->field, &c->field_bytes, in_bytes))) return rc;
        cudaError_t e = copy_async(c, c->field, data, in_bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_status(e);
        U.links = c->field;
        if (prec != data_dtype) {
            if ((rc = grow(&c->field2, &c->field2_bytes, (size_t)flue_field_bytes(NT, NX, NY, NZ, prec)))) return rc;
            if ((rc = flue_pack_field(c->field, data_dtype, st, NT, NX, NY, NZ, c->field2, prec, 0, c->st))) return rc;
            U.links = c->field2;
        }
    }
    if ((rc = ensure_ws(c, FLUE_OP_MAGNETIC_FORCE, U))) return rc;
    void* force_out = nullptr;
    void* grad_dst = nullptr;  // where the gradient in the data's dtype ends up on the device
    if (grad) {
        if (d_grad) {
            grad_dst = d_grad;
        } else {
            if ((rc = grow(&c->out, &c->out_bytes, in_bytes))) return rc;
            grad_dst = c->out;
        }
        force_out = grad_dst;
        if (widen) {
            // FP32 gradient first, in c->field (its complex128 input has been
            // packed into c->field2 by now), then widened into grad_dst
            if ((rc = grow(&c->field, &c->field_bytes, (size_t)flue_field_bytes(NT, NX, NY, NZ, FLUE_C64)))) return rc;
            force_out = c->field;
        }
    }
    if ((rc = flue_magnetic_force(&U, c->scal, force_out, force_form, c->ws, c->ws_bytes, c->st))) return rc;
    if (grad && widen) {
        const FieldRef G{force_out, make_geom(NT, NX, NY, NZ), FLUE_C64};
        cudaError_t e = launch_unpack(G, grad_dst, FLUE_C128, c->st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (grad && !d_grad) {
        cudaError_t e = copy_async(c, grad, c->out, in_bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_status(e);
    }
    return fetch(c, B, c->scal, sizeof(double));
}

void flue_release_host_cache(void) {
    std::lock_guard<std::mutex> lk(g_cache_mtx);
    for (DevCache* c : g_caches) {
        if (!c) continue;
        std::lock_guard<std::mutex> lk2(c->mtx);
        if (c->field) cudaFree(c->field);
        if (c->field2) cudaFree(c->field2);
        if (c->ws) cudaFree(c->ws);
        if (c->out) cudaFree(c->out);
        c->field = c->field2 = c->ws = c->out = nullptr;
        c->field_bytes = c->field2_bytes = c->ws_bytes = c->out_bytes = 0;
        for (int j = 0; j < DevCache::kPipeSlots; ++j) {
            if (c->slot[j]) cudaFree(c->slot[j]);
            c->slot[j] = nullptr;
            c->slot_bytes[j] = 0;
        }
        if (c->stage) cudaFree(c->stage);
        if (c->ostage) cudaFree(c->ostage);
        c->stage = c->ostage = nullptr;
        c->stage_bytes = c->ostage_bytes = 0;
    }
}

}  // extern "C"

namespace flue {
FLUE_OOB_READER(capi)
}  // namespace flue
