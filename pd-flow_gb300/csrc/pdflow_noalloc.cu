// pdflow_solve_pair_noalloc: a single-pair solve whose scratch memory is a
// fixed array compiled into this library, for callers that cannot allocate
// device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not wanted
// once the program is up, e.g. a real-time or safety-critical camera loop
// whose memory budget is fixed at start-up, a plugin inside a host framework
// that owns every device allocation, or a process whose allocator state must
// not change between frames.  The regular entry points (pdflow_create and
// friends) allocate one arena per handle; this one allocates nothing.
//
// The scratch is a file-scope __device__ array of kScratchBytes (12 MiB).  This
// translation unit has no kernels, so under CUDA's default lazy module loading
// its module (and with it the array) is loaded on a device by the first call's
// cudaGetSymbolAddress; from then (with CUDA_MODULE_LOADING=EAGER, from context
// creation) the GPU holds the 12 MiB until the process exits.  It fits 320x240
// frames with rows <= 120 (about 8.8 MB of pyramid and level buffers);
// larger configurations are rejected with PDFLOW_ERR_ARG.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the first call on each device, with that
// device current, resolves the array's device address with
// cudaGetSymbolAddress and keeps it for later calls on that device.  Make that
// first call before any stream capture begins.
//
// Every call uses the same array and leaves its contents behind.  The only
// word that must start at zero (the device status word) is cleared by each
// call; every other byte of scratch is written before it is read.  Two calls
// that overlap on the GPU (different streams, or host threads that do not
// serialise their calls) race on the array and corrupt each other's results:
// serialise them.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/pdflow.h"
#include "pdflow_internal.h"
#include "pdflow_iterate.cuh"
#include "pdflow_kernels.cuh"

namespace {

constexpr size_t kScratchBytes = size_t(12) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};   // device address of g_scratch, per device
int g_num_sms[kMaxDevices] = {};
// Records the failure for pdflow_last_error and returns `code`.
int fail(int code, const char* what, cudaError_t e = cudaSuccess)
{
    char buf[384];
    if (e != cudaSuccess)
        std::snprintf(buf, sizeof buf, "pdflow_solve_pair_noalloc: %s: %s", what, cudaGetErrorString(e));
    else
        std::snprintf(buf, sizeof buf, "pdflow_solve_pair_noalloc: %s", what);
    pdflow::set_last_error(buf);
    return code;
}

unsigned log2u(unsigned x)
{
    unsigned l = 0;
    while (x > 1) {
        x >>= 1;
        ++l;
    }
    return l;
}

// One-time set-up of the current device: its sm_103 check, the kernels'
// launch attributes and the device address of the scratch array.
int setup_device(int dev, void** scratch, int* num_sms)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_addr[dev]) {
        *scratch = g_scratch_addr[dev];
        *num_sms = g_num_sms[dev];
        return PDFLOW_OK;
    }
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return fail(PDFLOW_ERR_CUDA, "cudaGetDeviceProperties", e);
    if (!(prop.major == 10 && prop.minor == 3)) return fail(PDFLOW_ERR_NO_DEVICE, "needs an sm_103 (GB300) device");
    e = pdflow::prepare_iterate();
    if (e == cudaSuccess) e = pdflow::prepare_tiles();
    if (e == cudaSuccess) e = pdflow::prepare_tiles2();
    if (e != cudaSuccess) return fail(PDFLOW_ERR_CUDA, "kernel attributes", e);
    void* addr = nullptr;
    e = cudaGetSymbolAddress(&addr, g_scratch);
    if (e != cudaSuccess || addr == nullptr) return fail(PDFLOW_ERR_CUDA, "cudaGetSymbolAddress(scratch)", e);
    g_scratch_addr[dev] = addr;
    g_num_sms[dev] = prop.multiProcessorCount;
    *scratch = addr;
    *num_sms = prop.multiProcessorCount;
    return PDFLOW_OK;
}

}  // namespace

extern "C" {

int pdflow_solve_pair_noalloc(unsigned rows, unsigned width, unsigned height, const pdflow_params* params,
                              const uint8_t* d_intensity1, const uint16_t* d_depth1, const uint8_t* d_intensity2,
                              const uint16_t* d_depth2, float* d_dx, float* d_dy, float* d_dz, void* stream)
{
    if (!d_intensity1 || !d_depth1 || !d_intensity2 || !d_depth2 || !d_dx || !d_dy || !d_dz)
        return fail(PDFLOW_ERR_ARG, "null pointer argument");
    if (!(rows == 15 || rows == 30 || rows == 60 || rows == 120 || rows == 240 || rows == 480))
        return fail(PDFLOW_ERR_ARG, "rows must be one of 15,30,60,120,240,480");
    if (!((width == 640 && height == 480) || (width == 320 && height == 240)))
        return fail(PDFLOW_ERR_ARG, "image must be 640x480 or 320x240");
    const unsigned cols = rows * 320 / 240;
    if (cols > width) return fail(PDFLOW_ERR_ARG, "rows exceed the image resolution");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(PDFLOW_ERR_CUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return fail(PDFLOW_ERR_ARG, "device index out of range");
    void* scratch = nullptr;
    int num_sms = 0;
    int rc = setup_device(dev, &scratch, &num_sms);
    if (rc != PDFLOW_OK) return rc;

    // A handle that lives on this stack frame; its buffers are carved from the
    // static scratch array instead of an allocation.
    pdflow_solver s;
    s.device = dev;
    s.num_sms = num_sms;
    s.rows = rows;
    s.cols = cols;
    s.width = width;
    s.height = height;
    s.batch = 1;
    s.cam_mode = (height == 240) ? 2u : 1u;
    s.ctf_levels = log2u(rows / 15) + 1;
    s.pyr_levels = log2u(width / cols) + s.ctf_levels;
    if (params) s.prm = *params;
    else pdflow_default_params(rows, &s.prm);
    s.use_graph = 0;
    // Scalar tiles (form 2): they need no per-launch tensor maps and contain no
    // bounded wait, so nothing here can time out on the device; the paired
    // forms give the same bits (the tests compare against the regular entry
    // point, whose default is the paired 24x24 form).
    s.iter_form = 2;
    size_t need = 0;
    pdflow::carve_solver(&s, nullptr, &need);
    if (need > kScratchBytes) {
        char msg[200];
        std::snprintf(msg, sizeof msg,
                      "rows=%u with %ux%u frames needs %zu bytes of scratch; this entry point holds %zu "
                      "(320x240 frames with rows <= 120)",
                      rows, width, height, need, kScratchBytes);
        return fail(PDFLOW_ERR_ARG, msg);
    }
    pdflow::carve_solver(&s, static_cast<char*>(scratch), &need);
    s.dx = d_dx;   // the finest level's motion field goes straight to the caller
    s.dy = d_dy;
    s.dz = d_dz;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    s.stream = st;

    e = cudaMemsetAsync(s.status, 0, sizeof(unsigned), st);   // the one word that must start at zero
    if (e != cudaSuccess) return fail(PDFLOW_ERR_CUDA, "status reset", e);
    const uint8_t* img[2] = {d_intensity1, d_intensity2};
    const uint16_t* dep[2] = {d_depth1, d_depth2};
    for (int f = 0; f < 2; ++f) {
        s.new_slot ^= 1;
        e = pdflow::launch_decode_u16(img[f], dep[f], width, height, s.pyr[s.new_slot][0], s.prm.fovh, 1, 0, st);
        if (e != cudaSuccess) return fail(PDFLOW_ERR_CUDA, "decode launch", e);
        rc = pdflow::enqueue_pyramid(&s, st, 1);
        if (rc != PDFLOW_OK) return fail(rc, "pyramid launch");
    }
    s.frames = 2;
    rc = pdflow::enqueue_solve(&s, st, 1);
    if (rc != PDFLOW_OK) return rc;   // enqueue_solve recorded the error text
    return PDFLOW_OK;
}

}  // extern "C"
