// flue_internal.h -- host-side launchers shared between the kernel files and
// the C-ABI layer (capi.cu).  Every launcher is asynchronous on `stream`,
// validates nothing (capi.cu does that) and returns a cudaError_t.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "flue_common.cuh"

struct flue_field;

namespace flue {

struct FieldRef {
    const void* links;
    Geom g;
    int prec;
};

// Runs the statements with `T` (compute type) and `L` (link accessor) bound
// for the precision of FieldRef U.
#define FLUE_DISPATCH_LINKS(U, ...)                                              \
    do {                                                                         \
        if ((U).prec == PREC_C128) {                                             \
            using T = double;                                                    \
            FullLinks<double> L{(const double2*)(U).links, (U).g.V};             \
            __VA_ARGS__;                                                         \
        } else if ((U).prec == PREC_C64) {                                       \
            using T = float;                                                     \
            FullLinks<float> L{(const float2*)(U).links, (U).g.V};               \
            __VA_ARGS__;                                                         \
        } else {                                                                 \
            using T = float;                                                     \
            R12Links L{(const float4*)(U).links, (U).g.V};                       \
            __VA_ARGS__;                                                         \
        }                                                                        \
    } while (0)

// reduction finisher: out[j] = sum_i partial[j*nparts + i], j < nout
cudaError_t launch_finish_sums(const double* partial, int nparts, int nout, double* out, cudaStream_t st,
                               double scale = 1.0);

// layouts
// max_blocks > 0 caps the grid (the kernel is grid-strided); mu0 > 0 packs
// only the directions mu0..3 (the others are left as they are)
cudaError_t launch_pack(const void* src, int src_dtype, const int64_t strides[7], const Geom& g, void* dst, int dst_prec,
                        int reunitarise, cudaStream_t st, unsigned max_blocks = 0, int mu0 = 0);
cudaError_t launch_unpack(const FieldRef& U, void* dst, int dst_dtype, cudaStream_t st);
cudaError_t launch_matmul_batch(const void* l, const void* r, void* o, int64_t n, int dtype, int dagger, cudaStream_t st);
cudaError_t launch_fix_field(void* links, const Geom& g, int prec, cudaStream_t st);

// SM count of the current device (cudaDevAttrMultiProcessorCount), looked up
// once per device; 152 when no device answers (host-only size queries)
int device_sms();
// upper bound of every reduction grid below: 4 blocks per SM for up to 256
// SMs.  Workspaces hold this many partial-sum slots (the *_slots sizes), so
// a workspace sized on one device fits the grid on any other.
constexpr int kMaxRedBlocks = 1024;

// observables.  *_blocks is the launch grid on the current device (<=
// kMaxRedBlocks); the partial-sum scratch `part` needs *_slots(...) entries.
int plaquette_blocks(const Geom& g);
int plaquette_slots(const Geom& g);
int polyakov_slots(const Geom& g);
int wloop_slots(const Geom& g);
int meanlink_slots(const Geom& g);
cudaError_t launch_plaquette(const FieldRef& U, int mu0, int mu1, int nu1, double* part, double* out, cudaStream_t st);
int polyakov_blocks(const Geom& g);
cudaError_t launch_polyakov(const FieldRef& U, double* part, double* out2, cudaStream_t st);
int wloop_blocks(const Geom& g);
cudaError_t launch_wloop(const FieldRef& U, int tau, int mu, int nu, int nmu, int nnu, double* part, double* out,
                         cudaStream_t st);
cudaError_t launch_genericpath(const FieldRef& U, const int* path_host, int npath, const int* coord_host, void* out,
                               cudaStream_t st);
size_t wmunu_table_ws_bytes(const Geom& g, int prec, int rmax, int tmax);
cudaError_t launch_wmunu_table(const FieldRef& U, int mu, int nu, int rmax, int tmax, double* out, void* ws,
                               cudaStream_t st);
int meanlink_blocks(const Geom& g);
cudaError_t launch_meanlink(const FieldRef& U, const void* G, int g_dtype, double* part, double* out4, cudaStream_t st);

// field strength / energies (fmunu.cu, force.cu)
struct PlaneSet {
    int np;
    int mu[6], nu[6];  // 0-based directions
};
size_t energy_ws_bytes(const Geom& g, int prec, const PlaneSet& ps, bool with_force);
cudaError_t launch_fmunu(const FieldRef& U, int kind, int mu, int nu, void* out, void* ws, size_t ws_bytes,
                         cudaStream_t st);
cudaError_t launch_energy(const FieldRef& U, const PlaneSet& ps, double* out_E, void* force, int force_form, void* ws,
                          size_t ws_bytes, cudaStream_t st);
// T-slab form of launch_energy for plane sets without the time direction
// (B^2), where time slices are independent.  Part 1 (lines, forward, *out_E
// normalised by vfull, line cotangents when with_force) computes the slab of
// time slices [t0, t0 + nts) of field U (the whole field, or a packed slab
// with t0 = 0).  Part 2 (link cotangents, grid capped at max_blocks per
// direction when > 0) takes U with the slab's geometry (links unused) and
// writes the slab's gradient, normalised by vfull, at slices [t0, t0 + nts)
// of an array of time extent ntf (the whole lattice's gradient, or a chunk
// of time slices of it) as out_dtype: the compute dtype, or complex128
// (PREC_C128) from an FP32 computation.  Both use the same workspace, sized
// for the slab, and may run on different streams.
cudaError_t launch_energy_slab_fwd(const FieldRef& U, int t0, int nts, const PlaneSet& ps, int64_t vfull,
                                   double* out_E, bool with_force, void* ws, size_t ws_bytes, cudaStream_t st);
// skip_zero: the directions without a plane (zero gradient) are not written
// (the caller fills them).
cudaError_t launch_energy_slab_out(const FieldRef& U, const PlaneSet& ps, int64_t vfull, int ntf, int t0, void* force,
                                   int force_form, void* ws, size_t ws_bytes, unsigned max_blocks, cudaStream_t st,
                                   int out_dtype, bool skip_zero = false);
// launch_energy over nslab time slabs on nstream (<= 4) streams forked from
// st (plane sets without the time direction); workspace of
// energy_slabs_ws_bytes(...) bytes.  Results equal launch_energy's: the
// gradient bitwise, the energy up to the order of the FP64 partial sums.
size_t energy_slabs_ws_bytes(const Geom& g, int prec, const PlaneSet& ps, bool with_force, int nslab, int nstream);
cudaError_t launch_energy_slabs(const FieldRef& U, const PlaneSet& ps, double* out_E, void* force, int form, void* ws,
                                size_t ws_bytes, int nslab, int nstream, cudaStream_t st);
bool stage_timing_on();
int plaqforce_blocks(const Geom& g);
cudaError_t launch_plaquette_force(const FieldRef& U, double* part, double* out_S, void* force, int force_form,
                                   cudaStream_t st);

// out-of-bounds counters of the bounds-checked build, one per translation
// unit (read and cleared; 0 in the normal build)
unsigned oob_capi();
unsigned oob_ensemble();
unsigned oob_flow();
unsigned oob_force();
unsigned oob_noalloc();
unsigned oob_observables();
unsigned oob_propagator();

// text returned by flue_last_error_detail() on the calling thread
void set_error_detail(const char* msg);

// Argument checks shared by every device entry point (capi.cu): a NULL
// descriptor or links pointer, an unknown precision, bad extents and a links
// pointer off its element alignment (8 bytes for C64, 16 for C128 / R12) are
// refused with a status code and a detail text before anything is launched.
bool dims_ok(int nt, int nx, int ny, int nz);
bool prec_ok(int p);
int check_field(const ::flue_field* U, FieldRef* out);
// FLUE_OK for cudaSuccess, else FLUE_ERR_CUDA with the error's name and text
// as the detail
int cuda_status(cudaError_t e);

// process-wide count of kernel launches (flue_kernel_launches); every launch
// site calls it as `note_launch(), kernel<<<...>>>(...)`
void note_launch(int n = 1);

cudaError_t stage_timing_enable(int on);
cudaError_t stage_times(double* ms, int maxn, int* n);

// Wilson flow (flow.cu)
size_t wflow_ws_bytes(const Geom& g);
cudaError_t launch_wflow_step(void* links, const Geom& g, int prec, double eps, void* ws, cudaStream_t st);

// gauge transformation and gluon propagator (propagator.cu)
cudaError_t launch_gauge_transform(const FieldRef& U, const void* G, int g_dtype, cudaStream_t st);
size_t gluon_prop_ws_bytes(const Geom& g, int prec);
cudaError_t launch_gluon_propagator(const FieldRef& U, double xi, int mu_start, double* D, void* ws, size_t ws_bytes,
                                    cudaStream_t st);

}  // namespace flue
