// An L_p product entry point that allocates no device memory.
//
// Who needs it: callers that may not allocate on the device at the moment they compute, e.g. a host
// process whose device memory is handed out by an admission controller that accounts every byte up front
// (the solver's serving loop runs against a fixed HBM budget), or a latency-critical caller for which
// cudaMalloc's implicit device-wide synchronisation would stall other streams' work.  Every other entry
// point of this library allocates its FFT scratch per call (or per workspace); this one takes it from a
// fixed array compiled into the library instead.
//
// The scratch is a file-scope __device__ array of GT_LP_NOALLOC_SCRATCH_BYTES (32 MiB): every GPU that loads
// the library holds it until the process exits.  Host code cannot use the array's name as a device address,
// so its address is looked up with cudaGetSymbolAddress once per device, the first time this entry point
// runs with that device current, and cached; make that first call before any stream capture begins.
// The geometry's own device must be current: a call made with another device current is refused, since it
// would pair the geometry's buffers with that device's copy of the array.
// Every call uses the same array: two calls whose kernels overlap on the GPU (other streams, other host
// threads) race on it.  Nothing in it has to start at zero: the row pass writes every entry the column and
// inverse-row passes read.
#include "../../include/gt_gb300.h"
#include "common.cuh"

#include <exception>
#include <mutex>
#include <new>
#include <string>

struct gt_geometry;

namespace gt {
size_t lp_scratch_bytes(const gt_geometry* G, int ncol);
int geometry_device(const gt_geometry* G);
void lp_with_scratch(gt_geometry* G, int ncol, const c64* x, c64* y, void* scratch, cudaStream_t st);
void set_error(const std::string& s);
}  // namespace gt

static __device__ __align__(256) unsigned char g_lp_scratch[GT_LP_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_lock;

// The scratch array's device address on the current device (looked up once per device).
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_lock);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_lp_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}
}  // namespace

extern "C" int gt_lp_product_noalloc(gt_geometry* g, int32_t n_cols, const void* x_device, void* y_device,
                                     void* stream) {
    try {
        if (!g || n_cols < 1 || !x_device || !y_device) {
            gt::set_error("gt_lp_product_noalloc: null geometry or buffer, or n_cols < 1");
            return GT_INVALID_ARGUMENT;
        }
        const size_t need = gt::lp_scratch_bytes(g, n_cols);
        if (need > (size_t)GT_LP_NOALLOC_SCRATCH_BYTES) {
            gt::set_error("gt_lp_product_noalloc: " + std::to_string(n_cols) + " columns need " +
                          std::to_string(need) + " bytes of scratch, more than the fixed " +
                          std::to_string((size_t)GT_LP_NOALLOC_SCRATCH_BYTES) +
                          " bytes; pass fewer columns per call");
            return GT_INVALID_ARGUMENT;
        }
        int dev = -1;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) {
            gt::set_error(std::string("gt_lp_product_noalloc: cudaGetDevice failed: ") + cudaGetErrorString(e));
            return GT_DEVICE_ERROR;
        }
        if (dev != gt::geometry_device(g)) {
            gt::set_error("gt_lp_product_noalloc: the geometry lives on device " +
                          std::to_string(gt::geometry_device(g)) + " but device " + std::to_string(dev) +
                          " is current; make the geometry's device current");
            return GT_INVALID_ARGUMENT;
        }
        void* scratch = nullptr;
        e = scratch_address(&scratch);
        if (e != cudaSuccess) {
            gt::set_error(std::string("gt_lp_product_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
            return GT_DEVICE_ERROR;
        }
        gt::lp_with_scratch(g, n_cols, static_cast<const gt::c64*>(x_device), static_cast<gt::c64*>(y_device), scratch,
                            (cudaStream_t)stream);
        return GT_OK;
    } catch (const gt::CudaError& e) {
        gt::set_error(std::string("gt_lp_product_noalloc: ") + cudaGetErrorString(e.code) + " (" + e.where + ")");
        return e.code == cudaErrorMemoryAllocation ? GT_OUT_OF_MEMORY : GT_DEVICE_ERROR;
    } catch (const std::bad_alloc&) {
        gt::set_error("gt_lp_product_noalloc: host allocation failed");
        return GT_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        gt::set_error(std::string("gt_lp_product_noalloc: ") + e.what());
        return GT_INVALID_ARGUMENT;
    } catch (...) {
        gt::set_error("gt_lp_product_noalloc: unknown failure");
        return GT_DEVICE_ERROR;
    }
}
