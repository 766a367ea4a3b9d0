// Workspace-free backward transform (k -> x) of one FP64 field.
//
// Some callers cannot hand this library a workspace: an application whose
// device memory is owned by its own pool allocator and that forbids any other
// device allocation, code that must not pay cudaMalloc's implicit
// device-wide synchronisation inside a latency-critical loop, or a foreign
// host language that can pass arrays it already has but has no device
// allocator of its own.  For them dd_fft_c2r_noalloc runs the same transform
// as dd_fft_c2r with its intermediates in a static device buffer that is part
// of the library image, so the call allocates nothing.
//
// Limits and rules, for the caller:
//  * The buffer holds DD_NOALLOC_SCRATCH_BYTES (4 MiB).  That covers one FP64
//    field up to 64^3 in 3D and up to 512^2 in 2D, with or without 2/3
//    dealiasing (the Nyquist modes are never kept, so a 64^3 plan needs at
//    most 4.16 MB, 2.4 MB with 2/3 dealiasing); larger grids are rejected
//    with DD_ERR_UNSUPPORTED and a message giving the bytes they need.
//  * Every GPU that loads the library holds the 4 MiB until the process exits.
//  * Every call looks up the buffer's device address on the current device
//    (cudaGetSymbolAddress, a query that allocates nothing), so a device
//    reset between calls is harmless.  The first call on a device may load
//    the library's device code there; make that first call before any
//    stream capture.
//  * All calls share the one buffer, and it keeps whatever the last call
//    left in it.  Nothing in it has to start at zero: every scratch entry the
//    transform reads was written earlier in the same call.  Calls whose GPU
//    work overlaps (different streams, or different host threads without
//    ordering) race on the buffer; serialise them on one stream.
//  * The plan must belong to the current device: a plan made on another
//    device is rejected with DD_ERR_INVALID (its tables live there).
#include "dd_common.cuh"
#include "plan.cuh"

#define DD_NOALLOC_SCRATCH_BYTES (4u << 20)

static __device__ __align__(256) unsigned char dd_noalloc_scratch[DD_NOALLOC_SCRATCH_BYTES];

namespace {
// Device address of dd_noalloc_scratch on the current device.  In host code
// the symbol's name is only a host-side stand-in, never a device address.
int scratch_address(const dd_plan* plan, void** out) {
    int dev = 0;
    DD_CUDA(cudaGetDevice(&dev));
    DD_CHECK_ARG(plan->device == dev,
                 "dd_fft_c2r_noalloc: the plan belongs to device %d but device %d is current", plan->device, dev);
    void* p = nullptr;
    DD_CUDA(cudaGetSymbolAddress(&p, dd_noalloc_scratch));
    *out = p;
    return DD_OK;
}
}  // namespace

extern "C" int dd_fft_c2r_noalloc(const dd_plan* plan, const void* k, double* x, void* stream) {
    DD_CHECK_ARG(plan && k && x, "dd_fft_c2r_noalloc: null pointer");
    size_t need = 0;
    DD_TRY(dd_plan_workspace_size(plan, 1, DD_FP64, &need));
    DD_CHECK_SUPPORTED(need <= DD_NOALLOC_SCRATCH_BYTES,
                       "dd_fft_c2r_noalloc: this grid needs %zu bytes of scratch, more than the %u-byte "
                       "static buffer; use dd_fft_c2r with a caller-provided workspace",
                       need, (unsigned)DD_NOALLOC_SCRATCH_BYTES);
    void* scratch = nullptr;
    DD_TRY(scratch_address(plan, &scratch));
    const void* kin[1] = {k};
    double* xout[1] = {x};
    return dd_fft_c2r(plan, 1, kin, xout, DD_FP64, scratch, DD_NOALLOC_SCRATCH_BYTES, stream);
}
