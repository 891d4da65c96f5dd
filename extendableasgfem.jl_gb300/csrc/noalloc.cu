// Mean-based preconditioner on device vectors with no device allocation.
//
// This entry point has no counterpart in the reference package.  It exists for
// callers that must not allocate device memory at the moment they apply the
// preconditioner: for example a Julia session whose CUDA.jl memory pool has
// already reserved the GPU, an application that runs under a fixed
// device-memory budget, or a time-critical loop where a cudaMalloc (which can
// synchronise the device) is not acceptable.  The caller passes the input and
// output vectors (device layout, see sgfem_device_layout); the intermediate
// buffer of the three sine-transform passes lives in the array below, which
// every GPU that loads the library holds until the process exits.
#include <atomic>
#include <string>

#include "sgfem_internal.h"

// Largest intermediate buffer (n_dev * ld elements of the chosen precision).
static constexpr size_t kStaticScratchBytes = (size_t)SGFEM_STATIC_SCRATCH_BYTES;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
// device address of g_static_scratch, looked up once per device; host threads
// that make their first call on one device at the same time may both look it
// up, and both store the same address
std::atomic<void*> g_scratch_addr[kMaxDevices];

int scratch_address(sgfem_context* ctx, void** out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "static scratch: device index out of range");
    void* p = g_scratch_addr[ctx->device].load(std::memory_order_acquire);
    if (!p) {
        // the device is current (set by the caller of this function)
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return sg_cuda_fail(ctx, e, "cudaGetSymbolAddress(g_static_scratch)");
        g_scratch_addr[ctx->device].store(p, std::memory_order_release);
    }
    *out = p;
    return SGFEM_OK;
}

}  // namespace

extern "C" int sgfem_precondition_device_static(sgfem_context* ctx, const void* r_dev, void* z_dev, int precision) {
    SG_TRY(sg_check_ready(ctx));
    if (!r_dev || !z_dev) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    if (precision != SGFEM_FP64 && precision != SGFEM_FP32)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "precision must be SGFEM_FP64 or SGFEM_FP32");
    if (!ctx->lattice)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED,
                       "lattice preconditioner unavailable (dofs do not form a power-of-two lattice)");
    const size_t need = sg_vec_bytes(ctx, precision);
    if (need > kStaticScratchBytes)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT,
                       "sgfem_precondition_device_static: the vector needs " + std::to_string(need) +
                           " bytes of scratch, more than the static maximum of " +
                           std::to_string(kStaticScratchBytes) + " bytes");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    void* scratch = nullptr;
    SG_TRY(scratch_address(ctx, &scratch));
    // boundary rows of z are zero; the passes write every interior row of the
    // scratch before reading it, so the scratch needs no clearing
    SG_CUDA(ctx, cudaMemsetAsync(z_dev, 0, need, ctx->stream));
    SG_TRY(sg_lat_pass_x(ctx, precision, r_dev, scratch, nullptr));
    SG_TRY(sg_lat_pass_y(ctx, precision, scratch, nullptr, nullptr, nullptr));
    SG_TRY(sg_lat_pass_xinv(ctx, precision, scratch, z_dev, 0, nullptr));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SGFEM_OK;
}
