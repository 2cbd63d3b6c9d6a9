/*
 * flue_gb300.h -- C ABI of the GB300 (sm_103a) implementation of FLUE's
 * gluonic-observable path.
 *
 * This ABI replaces, for the Wilson-loop / field-strength path, the f2py-wrapped
 * Fortran shim c_wrapper/FLUE_c.f90 of the reference (RJaBi/FLUE_Lat), whose
 * module subroutines take ISO_C_BINDING kinds and Fortran-ordered arrays.
 * Nothing here uses C++ or torch types.  Two tiers:
 *
 *  1. Host-buffer entry points (suffix _c).  They take exactly the arguments
 *     of the reference routine they replace: the gauge field is the caller's
 *     host array complex(C_DOUBLE) data(NT,NX,NY,NZ,4,3,3) in Fortran order
 *     (src/wloops.F90:60), directions / coordinates / path entries are
 *     1-based, intent(out) values are written through pointers.  Each call
 *     copies the field to the GPU, runs the kernels and copies the result
 *     back before it returns (library-owned device buffers, reused between
 *     calls; one internal stream per device; calls are serialised).
 *
 *  2. Device entry points.  They work on a flue_field that already lives in
 *     GPU memory and are asynchronous on the caller's CUDA stream (`stream`
 *     is a cudaStream_t, NULL = legacy default stream).  Scalar results are
 *     written to DEVICE doubles.  Scratch memory is supplied by the caller
 *     (`ws`, `ws_bytes`); flue_workspace_bytes() gives the size.  Nothing in
 *     this tier allocates memory.
 *
 * Every function returns a status code (FLUE_OK = 0) and never exits,
 * traps or aborts; flue_strerror() describes a code.
 *
 * Device field layouts (flue_field.prec):
 *   FLUE_C128, FLUE_C64: complex128 / complex64 in the reference's own
 *     Fortran order (NT,NX,NY,NZ,4,3,3): the complex element of site s =
 *     t + NT*(x + NX*(y + NY*z)), direction mu (0..3 = t,x,y,z), row a,
 *     column b (0-based) is at s + V*(mu + 4*(a + 3*b)), V = NT*NX*NY*NZ.
 *     This is already site-fastest structure-of-arrays, so a field read
 *     with f2py / Fortran / numpy(order='F') is used with no re-layout.
 *   FLUE_R12: reconstruct-12 single precision: float4 (mu,k) of site s at
 *     s + V*(k + 3*mu), k = 0: (U00,U01), 1: (U02,U10), 2: (U11,U12); the
 *     third row is conj(row0 x row1) (src/gaugeIO/ILDG_bin.f90:120-146).
 * Arithmetic: FLUE_C128 fields are computed in FP64; FLUE_C64 and FLUE_R12
 * fields in FP32 with every global sum accumulated in FP64.
 */
#ifndef FLUE_GB300_H
#define FLUE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FLUE_OK 0
#define FLUE_ERR_ARG 1       /* bad argument value (direction, path, NULL) */
#define FLUE_ERR_SHAPE 2     /* bad lattice extents                         */
#define FLUE_ERR_DTYPE 3     /* unknown precision / dtype                   */
#define FLUE_ERR_LAYOUT 4    /* unsupported strides / alignment             */
#define FLUE_ERR_CUDA 5      /* a CUDA runtime call failed                  */
#define FLUE_ERR_TIMEOUT 6   /* a bounded device wait gave up               */
#define FLUE_ERR_WORKSPACE 7 /* ws_bytes smaller than required             */
#define FLUE_ERR_NOMEM 8     /* device allocation failed (host tier only)  */

/* ---- precisions ---------------------------------------------------------- */
#define FLUE_C128 0
#define FLUE_C64 1
#define FLUE_R12 2

/* ---- force forms --------------------------------------------------------- */
#define FLUE_FORCE_LIE 0    /* G = sum_a T^a d/dh O(e^{hT^a}U) = -1/2 TA(U N), T^a = i lambda^a/2 */
#define FLUE_FORCE_EUCLID 1 /* dO/dRe U + i dO/dIm U = N^+ (the torch.autograd convention)       */

/* ---- F_munu kinds -------------------------------------------------------- */
#define FLUE_FMUNU_CLOVER 0
#define FLUE_FMUNU_LOOP5 1

/* ---- workspace query operations ------------------------------------------ */
#define FLUE_OP_PLAQUETTE 0
#define FLUE_OP_POLYAKOV 1
#define FLUE_OP_WMUNU 2
#define FLUE_OP_FMUNU 3
#define FLUE_OP_MAGNETIC 4       /* B^2 forward only                   */
#define FLUE_OP_MAGNETIC_FORCE 5 /* B^2 forward + backward             */
#define FLUE_OP_ENERGY_FORCE 6   /* 5-loop energy, all six planes, + backward */
#define FLUE_OP_PLAQUETTE_FORCE 7
#define FLUE_OP_MEANLINK 8
#define FLUE_OP_WFLOW 9
#define FLUE_OP_GLUON_PROP 10    /* scalar gluon propagator (FFT buffers + cuFFT work area) */

typedef struct flue_field {
    const void *links; /* device pointer, layout given by prec */
    int32_t nt, nx, ny, nz;
    int32_t prec;
} flue_field;

const char *flue_strerror(int status);
int flue_abi_version(void);
/* bytes of a device field of this size and precision */
int64_t flue_field_bytes(int nt, int nx, int ny, int nz, int prec);
/* scratch bytes needed by the device entry point `op` (0 if none) */
size_t flue_workspace_bytes(int op, int nt, int nx, int ny, int nz, int prec);
/* Detail text of the last failure on the calling thread. */
const char *flue_last_error_detail(void);
/* Per-stage device timing of the energy / B^2 pipeline, the counterpart of
 * the `time` out-arguments that the reference fills from its stopwatch
 * (src/wloops.F90:122-125).  flue_stage_timing(1) makes later energy calls
 * record CUDA events between their stages (lines, forward, line cotangents,
 * link cotangents); flue_stage_times() waits for the last call and writes
 * up to max_stages durations in ms.  Process-wide, one device. */
int flue_stage_timing(int enable);
int flue_stage_times(double *ms, int max_stages, int *n_stages);
/* Number of GPU kernels this library has launched in this process (all
 * devices; a replayed ensemble graph counts its two kernels).  For launch
 * accounting by benchmarks and tests; no reference counterpart. */
uint64_t flue_kernel_launches(void);
/* Bounds-checked build only (compiled with -DFLUE_BOUNDS_CHECK=1): the number
 * of out-of-range indices the kernels' accessors met (and skipped) since the
 * last call; -1 in a normal build.  No reference counterpart. */
int64_t flue_bounds_errors(void);

/* ======================================================================== */
/* Tier 2: device entry points                                              */
/* ======================================================================== */

/* Re-layout a device array of links, complex128 (src_dtype FLUE_C128) or
 * complex64 (FLUE_C64), with element (t,x,y,z,mu,a,b) at
 * sum_k idx_k * strides[k] (strides in complex elements), into a device
 * field of precision dst_prec.  reunitarise != 0 applies FixSU3Matrix
 * (src/gaugeIO/ILDG_bin.f90:138-151) to every link on the way, in FP64.
 * Replaces the transpose + FixSU3Matrix tail of the gauge readers
 * (src/gaugeIO/ILDG_bin.f90:55-56, src/gaugeIO/openqcdfileio_standalone.f90:76-84). */
int flue_pack_field(const void *src, int src_dtype, const int64_t strides[7], int nt, int nx, int ny, int nz,
                    void *dst, int dst_prec, int reunitarise, void *stream);
/* Expand a device field into the reference layout, complex128 or complex64. */
int flue_unpack_field(const flue_field *U, void *dst, int dst_dtype, void *stream);
/* FixSU3Matrix on every link of a device field, in place. */
int flue_reunitarise_field(const flue_field *U, void *stream);

/* Batched MultiplyMatMat (src/SU3MatrixOps.f90:19-37, exposed by
 * c_wrapper/FLUE_c.f90:31-36); dagger != 0 gives MultiplyMatdagMatdag
 * (:39-58), which computes left^+ right^+.  n matrices of 9 complex each,
 * Fortran order (a + 3b). */
int flue_multiplymatmat_batch(const void *left, const void *right, void *out, int64_t n, int dtype, int dagger,
                              void *stream);

/* plaquette / genPlaquette (src/wloops.F90:915-1017 / :59-127): d_sum[0] =
 * sum over planes mu in [muStart,muEnd], nu in (mu,nuEnd] and all sites of
 * Re Tr P_munu (no 1/3).  nP = V * #planes. */
int flue_plaquette(const flue_field *U, int muStart, int muEnd, int nuEnd, double *d_sum, void *ws, size_t ws_bytes,
                   void *stream);
/* polyakov (src/wloops.F90:1019-1069): d_sum[0] = sum_x Re Tr prod_t U_1,
 * d_sum[1] = the imaginary part.  nP = NX*NY*NZ. */
int flue_polyakov(const flue_field *U, double *d_sum2, void *ws, size_t ws_bytes, void *stream);
/* The W_munu table: d_out[(R-1)*tmax + (T-1)] = wmunu(mu, nu, R, T)
 * (src/wloops.F90:679-791, whole lattice, normalised by V) for every
 * R <= rmax, T <= tmax (1..64), from lines built once per site instead of
 * one call per (R, T); scratch flue_wmunu_table_bytes(...) bytes. */
size_t flue_wmunu_table_bytes(int nt, int nx, int ny, int nz, int prec, int rmax, int tmax);
int flue_wmunu_table(const flue_field *U, int mu, int nu, int rmax, int tmax, double *d_out, void *ws,
                     size_t ws_bytes, void *stream);
/* wmunu (src/wloops.F90:679-791) for tau = 0, wmunutau (:567-677) for
 * tau in 1..NT: d_val[0] = the MEAN nMu x nNu loop (divided by V or NX*NY*NZ). */
int flue_wmunu(const flue_field *U, int tau, int mu, int nu, int nMu, int nNu, double *d_val, void *ws,
               size_t ws_bytes, void *stream);
/* genericPath (src/wloops.F90:20-57): transpose of the ordered product of
 * links along `path` (host array of npath <= 256 entries +-1..+-4).
 * coordBase (host, 1-based) != NULL: one site, d_out = 9 complex (Fortran
 * order); NULL: every site, d_out = (NT,NX,NY,NZ,3,3).  complex128 output
 * for FLUE_C128 fields, complex64 otherwise. */
int flue_genericpath(const flue_field *U, const int *coordBase, const int *path, int npath, void *d_out, void *stream);
/* cloverLoopMuNuCoord (kind FLUE_FMUNU_CLOVER, src/wloops.F90:129-199) or
 * Loop5MuNuCoord (FLUE_FMUNU_LOOP5, :201-432) for plane (mu,nu): d_out =
 * (NT,NX,NY,NZ,3,3), complex128 / complex64 as for genericpath. */
int flue_fmunu(const flue_field *U, int kind, int mu, int nu, void *d_out, void *ws, size_t ws_bytes, void *stream);
/* magnetic (src/wloops.F90:479-544): d_B[0] = B^2. */
int flue_magnetic(const flue_field *U, double *d_B, void *ws, size_t ws_bytes, void *stream);
/* B^2 (magnetic) and, when d_force != NULL, its gradient for all four
 * directions in the field layout (complex128 for FLUE_C128, complex64
 * otherwise; temporal links get 0).  No reference counterpart for the
 * gradient. */
int flue_magnetic_force(const flue_field *U, double *d_B, void *d_force, int force_form, void *ws, size_t ws_bytes,
                        void *stream);
/* Energy over an arbitrary set of 5-loop planes (1-based (mu,nu) pairs,
 * nplanes <= 6, each unordered plane at most once): d_E[0] =
 * -1/V sum_x sum_planes Re Tr(F F); gradient as for flue_magnetic_force. */
int flue_loop5_energy_force(const flue_field *U, const int *planes, int nplanes, double *d_E, void *d_force,
                            int force_form, void *ws, size_t ws_bytes, void *stream);
/* Wilson plaquette sum S = sum_{x,mu<nu} Re Tr P_munu(x) and its gradient. */
int flue_plaquette_force(const flue_field *U, double *d_S, void *d_force, int force_form, void *ws, size_t ws_bytes,
                         void *stream);
/* Landau-gauge mean link: d_sum4[mu-1] = sum_x Re Tr(G(x) U_mu(x) G(x+mu)^+)
 * for a device gauge transformation G of layout (NT,NX,NY,NZ,3,3)
 * (ReadGaugeTransformation_cola's result, src/gaugeIO/ILDG_bin.f90:65-105),
 * complex128 or complex64 (g_dtype). */
int flue_meanlink(const flue_field *U, const void *G, int g_dtype, double *d_sum4, void *ws, size_t ws_bytes,
                  void *stream);
/* One Luescher RK3 step of the Wilson flow with step eps, in place; the
 * field must be FLUE_C128 or FLUE_C64. */
int flue_wflow_step(const flue_field *U, double eps, void *ws, size_t ws_bytes, void *stream);
/* Gauge transformation in place: U_mu(x) <- G(x) U_mu(x) G(x+mu)^+ for a
 * device G of layout (NT,NX,NY,NZ,3,3), complex128 or complex64 (g_dtype);
 * applies the Landau-gauge transformation that ReadGaugeTransformation_cola
 * reads (src/gaugeIO/ILDG_bin.f90:65-105) before a propagator measurement.
 * G must be SU(3) (an R12 field keeps two rows). */
int flue_gauge_transform(const flue_field *U, const void *G, int g_dtype, void *stream);
/* Scalar gluon propagator on every lattice momentum (the observable that
 * src/gluonCalc/gluonProp.f90 works towards, defined as in hep-lat/9803105,
 * which that file cites; the reference's routines are unfinished):
 *   A_mu(x) = [U_mu(x) - U_mu(x)^+]/(2i) - trace/3,  A^a = Tr(A lambda^a),
 *   A^a_mu(q) = sum_x exp(-i q.x) A^a_mu(x),  q_mu = 2 pi n_mu / N_mu,
 *   D(q) = sum_{mu >= mu_start} w_mu sum_a |A^a_mu(q)|^2 / (8 n(q) V),
 * w_t = xi^2 (anisotropy, as gluonProp.f90:186-190), w_i = 1, n(0) = 4,
 * n(q != 0) = 3 (gluonProp.f90:208-236); mu_start = 0 sums all four
 * directions, 1 the spatial ones.  The phase exp(-i q_mu/2) of the
 * midpoint convention has modulus 1 and drops out.  d_D: FP64
 * (NT,NX,NY,NZ), index n_mu = 0..N_mu-1 (n_mu > N_mu/2: negative q).  The
 * field should be Landau-gauge fixed (flue_gauge_transform).  Transforms by
 * cuFFT in the field's compute precision; scratch flue_workspace_bytes(
 * FLUE_OP_GLUON_PROP, ...). */
int flue_gluon_propagator(const flue_field *U, double xi, int mu_start, double *d_D, void *ws, size_t ws_bytes,
                          void *stream);

/* ---- ensemble batching (no reference counterpart; the reference's
 * magnetic app loops over configurations one by one, app/magnetic.f90:109-140)
 *
 * Plaquettes, Polyakov loop and B^2 of up to thousands of device fields of
 * uneven volume (all of one precision) in ONE persistent launch.  The launch
 * is cooperative (every block resident; a grid of blocks_per_sm x SM blocks
 * of `block` threads, 128 or 256, reduced to what fits) and works through a
 * task list from an atomic counter: the 5-loop lines of a chunk of a time
 * slab, the line-based B^2 of a chunk (each waiting, with a bounded wait,
 * for its slab's lines), and plaquettes / Polyakov loops of tile_cols time
 * columns; a finisher sums each field's partials in list order.  A wait that
 * runs out (not met in a healthy run) makes every output NaN.  One
 * ensemble's evaluations share its counters and line buffers: they must not
 * overlap on the GPU (run them in order on one stream).
 * Per field the output holds 6 doubles: sum Re Tr P over spatial planes, over
 * temporal planes, sum Re Tr and Im Tr of the Polyakov loop, B^2 (divided by
 * V; 0 when with_b2 = 0), V.  create() allocates the task list, partials and
 * a ring of four slab-line buffers on the current device (library-owned;
 * FLUE_ENS_SLAB_SITES, read here, sets the sites per slab, default 2^17);
 * items() returns the number of tasks; capture() records memset + kernel +
 * finisher writing to d_out into a CUDA graph, replay() launches it.
 * tile_cols = 0 selects pipeline mode instead (block, blocks_per_sm unused):
 * per field the device entry points -- flue_plaquette (spatial, temporal),
 * flue_polyakov, flue_magnetic (line-based, time slabs) -- with one
 * library-owned workspace for the largest field, the same outputs; capture()
 * then runs one evaluation uncaptured first (the entry points set up their
 * library streams on first use) and records every field's kernels. */
typedef struct flue_ensemble flue_ensemble;
int flue_ensemble_create(flue_ensemble **e, const flue_field *fields, int nfields, int tile_cols, int block,
                         int blocks_per_sm, int with_b2);
int flue_ensemble_items(const flue_ensemble *e);
int flue_ensemble_run(flue_ensemble *e, double *d_out, void *stream);
int flue_ensemble_capture(flue_ensemble *e, double *d_out);
int flue_ensemble_replay(flue_ensemble *e, void *stream);
int flue_ensemble_destroy(flue_ensemble *e);

/* Allocation-free plaquette.  No counterpart in the reference.  Same result
 * as flue_plaquette (same kernel, bitwise the same sum) but without a
 * workspace argument: the per-block partial sums live in an 8 KiB array that
 * is part of the library's device image, so the call allocates nothing --
 * for callers that own all device memory themselves (a simulation measuring
 * the plaquette in its update loop through ISO_C_BINDING while its pool holds
 * the HBM, or a framework whose allocator this library cannot reach).  Limit:
 * 1024 partial sums; the plaquette launch never uses more than 608 blocks, so
 * every lattice the ABI accepts fits, and a larger need is refused with
 * FLUE_ERR_WORKSPACE.  The arguments are checked exactly as flue_plaquette
 * checks them (precision, extents, links alignment).  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and
 * keeps it; make that first call before any stream capture, and do not use
 * this entry point across a cudaDeviceReset in the same process (the module
 * can be reloaded at another address).  All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
int flue_plaquette_noalloc(const flue_field *U, int muStart, int muEnd, int nuEnd, double *d_sum, void *stream);

/* ======================================================================== */
/* Tier 1: host-buffer entry points (reference signatures)                  */
/* data: host complex128 (NT,NX,NY,NZ,4,3,3), Fortran order.                */
/* ======================================================================== */

/* plaquette(data, muStart, muEnd, nuEnd, sumTrP, nP, time), src/wloops.F90:915.
 * time = device time of the kernels in seconds. */
int flue_plaquette_c(const double *data, int NT, int NX, int NY, int NZ, int muStart, int muEnd, int nuEnd,
                     double *sumTrP, int *nP, double *time);
/* genPlaquette(data,NT,NX,NY,NZ,muStart,muEnd,nuEnd,sumTrP,nP,time), src/wloops.F90:59. */
int flue_genplaquette_c(const double *data, int NT, int NX, int NY, int NZ, int muStart, int muEnd, int nuEnd,
                        double *sumTrP, int *nP, double *time);
/* polyakov(data, sumTrP, nP, time), src/wloops.F90:1019. */
int flue_polyakov_c(const double *data, int NT, int NX, int NY, int NZ, double *sumTrP, int *nP, double *time);
/* genericPath(data, coordBase, path) -> U_xd(3,3), src/wloops.F90:20. */
int flue_genericpath_c(const double *data, int NT, int NX, int NY, int NZ, const int *coordBase, const int *path,
                       int npath, double *U_xd);
/* wmunu(data, mu, nu, nMu, nNu) -> loopVal, src/wloops.F90:679. */
int flue_wmunu_c(const double *data, int NT, int NX, int NY, int NZ, int mu, int nu, int nMu, int nNu,
                 double *loopVal);
/* wmunutau(data, tau, mu, nu, nMu, nNu) -> loopVal, src/wloops.F90:567. */
int flue_wmunutau_c(const double *data, int NT, int NX, int NY, int NZ, int tau, int mu, int nu, int nMu, int nNu,
                    double *loopVal);
/* cloverLoopMuNuCoord(data,NT,NX,NY,NZ,mu,nu) -> U_xd(NT,NX,NY,NZ,3,3), src/wloops.F90:129. */
int flue_cloverloopmunucoord_c(const double *data, int NT, int NX, int NY, int NZ, int mu, int nu, double *U_xd);
/* Loop5MuNuCoord(data,NT,NX,NY,NZ,mu,nu) -> U_xd(NT,NX,NY,NZ,3,3), src/wloops.F90:201. */
int flue_loop5munucoord_c(const double *data, int NT, int NX, int NY, int NZ, int mu, int nu, double *U_xd);
/* magnetic(data,NT,NX,NY,NZ) -> B, src/wloops.F90:479. */
int flue_magnetic_c(const double *data, int NT, int NX, int NY, int NZ, double *B);
/* MultiplyMatMat_c(MM, left, right), c_wrapper/FLUE_c.f90:31-36. */
int flue_multiplymatmat_c(double *MM, const double *left, const double *right);
/* FixSU3Matrix(U_x) in place, src/gaugeIO/ILDG_bin.f90:138. */
int flue_fixsu3matrix_c(double *U_x);
/* uzerobar (README.md:17; no reference code): u0[0..2] = plaquette u0 over
 * all planes (<ReTrP>/3)^(1/4), spatial (<ReTrP_ss>/3)^(1/4) and temporal
 * (<ReTrP_st>/3)^(1/2)/u0_s; u0[3..5] = Landau mean link <ReTr U'>/3 over
 * all, spatial and temporal links with U'_mu(x) = G(x) U_mu(x) G(x+mu)^+ when
 * G (host complex128 (NT,NX,NY,NZ,3,3), Fortran order) is given, else NaN. */
int flue_uzerobar_c(const double *data, int NT, int NX, int NY, int NZ, const double *G, double *u0);
/* scalarGluonProp_c (c_wrapper/FLUE_c.f90:9-16, src/gluonCalc/gluonProp.f90:17-112):
 * same arguments -- NS, NT, host complex128 U(NT,NS,NS,NS,4,3,3) in position
 * space, anisotropy xi -- and D the propagator of flue_gluon_propagator with
 * mu_start = 0, host FP64 of shape (NT,NS,NS,NS) (the reference declares
 * (NS,NS,NS,NS), which holds it only when NT = NS). */
int flue_scalargluonprop_c(int NS, int NT, const void *U, double xi, double *D);
/* B^2 forward + backward from host buffers: data is complex128
 * (data_dtype FLUE_C128) or complex64 (FLUE_C64), computed in precision
 * prec -- complex128 data in any precision (FP32 link products for FLUE_C64
 * and FLUE_R12, the field rounded on the GPU), complex64 data in FLUE_C64 or
 * FLUE_R12; grad (host, same layout and dtype as data) receives the gradient
 * of B^2 in form force_form. */
int flue_magnetic_force_c(const void *data, int data_dtype, int NT, int NX, int NY, int NZ, int prec, int force_form,
                          double *B, void *grad);
/* Release the library-owned device buffers of the host tier. */
void flue_release_host_cache(void);

#ifdef __cplusplus
}
#endif
#endif /* FLUE_GB300_H */
