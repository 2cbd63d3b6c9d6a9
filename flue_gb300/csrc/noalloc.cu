// noalloc.cu -- a plaquette entry point that allocates no memory at all.
//
// Who needs it: programs that own every byte of device memory themselves and
// cannot (or must not) let a library call cudaMalloc -- for example a lattice
// simulation that measures the plaquette inside its update loop through a
// Fortran ISO_C_BINDING interface while its own memory pool holds nearly all
// of HBM, or a host framework whose allocator is not reachable from this
// library.  cudaMalloc may fail there, or synchronise the device and fragment
// a pool that the caller manages.  flue_plaquette() needs a caller-supplied
// workspace for its per-block partial sums; this variant keeps them in a
// fixed device array that is part of the library image instead.
//
// The array is a file-scope __device__ object of FLUE_NOALLOC_SCRATCH_DOUBLES
// doubles (8 KiB).  Every GPU on which the library is loaded holds it until
// the process exits.  It is shared by all calls and keeps the contents of the
// last call; the kernel writes every slot it later reads, so nothing has to
// be cleared between calls.  Two calls whose work overlaps on the GPU (for
// example on two streams at once) race on the array and can both return
// wrong sums: serialise them.  The array's address is looked up on the first
// call on each device and kept, so this entry point must not be used across a
// cudaDeviceReset in the same process.
#include <mutex>

#include "../../include/flue_gb300.h"
#include "flue_internal.h"

#define FLUE_NOALLOC_SCRATCH_DOUBLES 1024

namespace {

static __device__ __align__(256) double g_noalloc_scratch[FLUE_NOALLOC_SCRATCH_DOUBLES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mtx;
double* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device.  Host code sees only a host-side stand-in for the symbol, so
// the address must come from cudaGetSymbolAddress.  The cached address is
// not refreshed: after cudaDeviceReset the module may load elsewhere, so the
// entry point must not be used across a device reset in one process.
cudaError_t scratch_on_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mtx);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int flue_plaquette_noalloc(const flue_field* U, int muStart, int muEnd, int nuEnd, double* d_sum,
                                      void* stream) {
    // the same validator as flue_plaquette: NULL pointers, precision,
    // extents and the links pointer's alignment are refused before launch
    flue::FieldRef F;
    int rc = flue::check_field(U, &F);
    if (rc) return rc;
    if (!d_sum) {
        flue::set_error_detail("flue_plaquette_noalloc: NULL output pointer");
        return FLUE_ERR_ARG;
    }
    if (muStart < 1 || muEnd > 4 || nuEnd > 4 || muStart > muEnd + 1 || nuEnd < 1) {
        flue::set_error_detail("flue_plaquette_noalloc: plane range out of 1..4");
        return FLUE_ERR_ARG;
    }
    // one FP64 partial per block of the plaquette kernel
    const int need = flue::plaquette_blocks(F.g);
    if (need > FLUE_NOALLOC_SCRATCH_DOUBLES) {
        flue::set_error_detail("flue_plaquette_noalloc: this lattice needs more partial-sum slots than the "
                               "built-in scratch array holds (1024); use flue_plaquette with a workspace");
        return FLUE_ERR_WORKSPACE;
    }
    double* scratch = nullptr;
    cudaError_t se = scratch_on_current_device(&scratch);
    if (se != cudaSuccess) {
        cudaGetLastError();
        flue::set_error_detail("flue_plaquette_noalloc: cudaGetSymbolAddress of the scratch array failed");
        return FLUE_ERR_CUDA;
    }
    return flue::cuda_status(
        flue::launch_plaquette(F, muStart - 1, muEnd - 1, nuEnd - 1, scratch, d_sum, (cudaStream_t)stream));
}

namespace flue {
FLUE_OOB_READER(noalloc)
}  // namespace flue
