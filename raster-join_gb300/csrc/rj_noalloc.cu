// rj_noalloc.cu -- raster join count that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: hosts that hand a plugin
// a fixed slice of GPU memory and account for every byte themselves, loops
// that must not stall on the device-wide synchronisation a first-time
// allocation can cause, and processes that already sit at the memory limit
// where a fresh allocation would fail in the middle of a query.  For them
// rj_raster_count_noalloc runs the bounded raster join (count per polygon)
// with every intermediate buffer -- the point canvas, the window-space
// vertices, the polygon-pass work lists -- carved out of one fixed,
// file-scope device array.  The caller provides the inputs and the output as
// device pointers.
//
// Limits (the array is sized for them; larger requests are rejected):
//   canvas           <= kNaMaxPixels pixels, one tile (no canvas tiling)
//   polygon vertices <= kNaMaxVerts
//   polygons         <= kNaMaxPolys
// Every GPU that loads the library holds the array (kNaScratchBytes) until
// the process exits.  All calls share it: calls that overlap on the GPU (on
// different streams, or from several host threads without ordering) race on
// it and produce wrong counts.  The first call on a device looks the array's
// address up for that device (cudaGetSymbolAddress); make that first call
// before capturing the stream into anything that records work.
// Errors: argument and size checks fail before any work is queued.  A CUDA
// error already pending on the calling thread when the call starts is
// reported (RJ_E_CUDA) and left pending, and nothing is queued; otherwise a
// CUDA error returned by the call comes from this call's own launches.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "rj_device.cuh"
#include "rj_launch.h"

namespace {

constexpr int kNaMaxRes = 2048;                                   // canvas side
constexpr size_t kNaMaxPixels = (size_t)kNaMaxRes * kNaMaxRes;
constexpr int kNaMaxVerts = 1 << 18;
constexpr int kNaMaxPolys = 1 << 16;
constexpr size_t kAlign = 256;

constexpr size_t align_up(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

// Layout of the array (each piece 256-byte aligned).
constexpr size_t kOffXf = 0;                                                    // 2 x float4
constexpr size_t kOffErr = align_up(kOffXf + 2 * sizeof(float4));               // int
constexpr size_t kOffCtr = align_up(kOffErr + sizeof(int));                     // unsigned
constexpr size_t kOffCanvas = align_up(kOffCtr + sizeof(unsigned));             // u32 per pixel
constexpr size_t kOffWv = align_up(kOffCanvas + kNaMaxPixels * sizeof(uint32_t));  // int2 per vertex
constexpr size_t kOffInfoA = align_up(kOffWv + (size_t)kNaMaxVerts * sizeof(int2));
constexpr size_t kOffInfoB = align_up(kOffInfoA + (size_t)kNaMaxPolys * sizeof(int4));
constexpr size_t kOffBands = align_up(kOffInfoB + (size_t)kNaMaxPolys * sizeof(int2));
constexpr size_t kOffBandStart = align_up(kOffBands + (size_t)kNaMaxPolys * sizeof(int));
constexpr size_t kOffScan = align_up(kOffBandStart + (size_t)(kNaMaxPolys + 1) * sizeof(int));
constexpr size_t kScanInts = 64;   // tile sums of a scan over <= kNaMaxPolys items
constexpr size_t kNaScratchBytes = align_up(kOffScan + kScanInts * sizeof(int));

static_assert(kNaScratchBytes < (24u << 20), "allocation-free scratch exceeds its 24 MiB budget");

}  // namespace

// The scratch array.  In host code its name is only a host-side stand-in:
// the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

namespace {

struct NaDevice {
    bool ready = false;
    unsigned char* ptr = nullptr;
    int sms = 1;
};
constexpr int kNaMaxDevices = 64;
NaDevice g_na_dev[kNaMaxDevices];
std::mutex g_na_mutex;

int na_fail(char* err, size_t errlen, int code, const char* msg) {
    if (err && errlen) {
        std::strncpy(err, msg, errlen - 1);
        err[errlen - 1] = '\0';
    }
    return code;
}

// Writes the canvas transform into the scratch array (no host staging).
__global__ void k_noalloc_xf(float4 col, float4 row, float4* dst) {
    dst[0] = col;
    dst[1] = row;
}

}  // namespace

using namespace rj;

extern "C" RJ_API int rj_raster_count_noalloc(const float* d_xy, uint64_t npoints, const float* d_verts,
                                              const int32_t* d_pindex, int32_t npolys, int32_t nverts,
                                              const double* bbox, double cell_size, unsigned long long* d_count,
                                              void* stream, char* err, size_t errlen) {
    if (err && errlen) err[0] = '\0';
    if (!d_xy && npoints) return na_fail(err, errlen, RJ_E_INVALID, "d_xy is null");
    if (!d_verts || !d_pindex || !d_count || !bbox) return na_fail(err, errlen, RJ_E_INVALID, "null argument");
    if (((uintptr_t)d_xy & 15) != 0) return na_fail(err, errlen, RJ_E_INVALID, "d_xy must be 16-byte aligned");
    if (npolys < 1 || npolys > kNaMaxPolys)
        return na_fail(err, errlen, RJ_E_INVALID, "npolys must be 1..65536 for the allocation-free join");
    if (nverts < 0 || nverts > kNaMaxVerts)
        return na_fail(err, errlen, RJ_E_INVALID, "nverts must be 0..262144 for the allocation-free join");
    const double dx = bbox[2] - bbox[0], dy = bbox[3] - bbox[1];
    if (!(dx > 0 && dy > 0)) return na_fail(err, errlen, RJ_E_INVALID, "empty bounds");
    if (!(cell_size > 0) || !std::isfinite(cell_size)) return na_fail(err, errlen, RJ_E_INVALID, "bad cell size");
    const double ax = std::ceil(dx / cell_size), ay = std::ceil(dy / cell_size);
    if (ax > kNaMaxRes || ay > kNaMaxRes)
        return na_fail(err, errlen, RJ_E_INVALID,
                       "canvas larger than 2048 x 2048 pixels: use rj_execute, or a larger cell size");
    const int resx = std::max(1, (int)ax), resy = std::max(1, (int)ay);
    // the polygon work-list scan's tile sums must fit their slice of the
    // array; checked before anything is queued on the caller's stream
    if (scan_tmp_ints(npolys) > (int)kScanInts)
        return na_fail(err, errlen, RJ_E_INVALID, "polygon work list exceeds the scratch array");
    // An error left pending by earlier work on this thread is not this call's:
    // report it and leave it pending for its owner, queueing nothing.
    {
        const cudaError_t prior = cudaPeekAtLastError();
        if (prior != cudaSuccess) {
            char msg[192];
            std::snprintf(msg, sizeof msg, "an earlier CUDA error is pending on this thread: %s",
                          cudaGetErrorString(prior));
            return na_fail(err, errlen, RJ_E_CUDA, msg);
        }
    }

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) {
        cudaGetLastError();
        return na_fail(err, errlen, RJ_E_CUDA, "no current CUDA device");
    }
    NaDevice& nd = g_na_dev[dev];
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!nd.ready) {
            // once per device, with that device current
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return na_fail(err, errlen, RJ_E_CUDA, "cudaGetSymbolAddress of the scratch array failed");
            }
            cudaDeviceGetAttribute(&nd.sms, cudaDevAttrMultiProcessorCount, dev);
            nd.ptr = (unsigned char*)p;
            nd.ready = true;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* base = nd.ptr;
    float4* xf = (float4*)(base + kOffXf);
    int* derr = (int*)(base + kOffErr);
    unsigned* ctr = (unsigned*)(base + kOffCtr);
    uint32_t* canvas = (uint32_t*)(base + kOffCanvas);
    int2* wv = (int2*)(base + kOffWv);
    const size_t npix = (size_t)resx * resy;

    // what must start at zero: the canvas, the counters and the output
    if (cudaMemsetAsync(canvas, 0, npix * sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(derr, 0, sizeof(int), st) != cudaSuccess ||
        cudaMemsetAsync(ctr, 0, sizeof(unsigned), st) != cudaSuccess ||
        cudaMemsetAsync(d_count, 0, sizeof(unsigned long long) * npolys, st) != cudaSuccess) {
        cudaGetLastError();
        return na_fail(err, errlen, RJ_E_CUDA, "cudaMemsetAsync failed");
    }
    // one canvas tile: the model-view-projection of the whole bounds
    const double ox = (bbox[2] + bbox[0]) / 2, hx = (bbox[2] - bbox[0]) / 2;
    const double oy = (bbox[3] + bbox[1]) / 2, hy = (bbox[3] - bbox[1]) / 2;
    const float sx = (float)(1.0 / hx), sy = (float)(1.0 / hy);
    const float4 col = make_float4(sx, sx * (float)(-ox), resx * 0.5f, (float)dx);
    const float4 row = make_float4(sy, sy * (float)(-oy), resy * 0.5f, (float)dy);
    k_noalloc_xf<<<1, 1, 0, st>>>(col, row, xf);
    launch_transform_vertices((const float2*)d_verts, nverts, xf, xf + 1, 1, 1, wv, nullptr, nd.sms, st);

    // point pass: counts into the canvas
    CanvasXf cx{};
    cx.colxf = xf;
    cx.rowxf = xf + 1;
    cx.splitx = cx.splity = 1;
    cx.resx = resx;
    cx.resy = resy;
    cx.lbx = (float)bbox[0];
    cx.lby = (float)bbox[1];
    cx.tdx = (float)dx;
    cx.tdy = (float)dy;
    cx.col0 = col;
    cx.row0 = row;
    PointArgs pa{};
    pa.xy = (const float2*)d_xy;
    pa.n = npoints;
    pa.P = 0;
    pa.err = derr;
    launch_raster_splat(pa, cx, canvas, nullptr, nd.sms, st);

    // polygon pass: sum the canvas over each polygon's covered pixels
    PolyPassArgs a{};
    a.wv = wv;
    a.pindex = d_pindex;
    a.P = npolys;
    a.V = nverts;
    a.T = 1;
    a.resx = resx;
    a.resy = resy;
    a.canvas_c = canvas;
    a.out_count = d_count;
    a.work_ctr = ctr;
    a.info_a = (int4*)(base + kOffInfoA);
    a.info_b = (int2*)(base + kOffInfoB);
    a.nbands = (int*)(base + kOffBands);
    a.band_start = (int*)(base + kOffBandStart);
    launch_poly_info(MODE_REDUCE, a, nd.sms, st);
    launch_exclusive_scan(a.nbands, (int*)(base + kOffBandStart), npolys, (int*)(base + kOffScan), st);
    launch_poly_pass(MODE_REDUCE, a, nd.sms, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(err, errlen, RJ_E_CUDA, cudaGetErrorString(e));
    return RJ_OK;
}
