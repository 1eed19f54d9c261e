// arc_noalloc.cu — arc_trace_frame_noalloc: the frame pass without any device allocation.
//
// Some callers cannot call cudaMalloc at the time they trace: a renderer that reserves all device
// memory up front and runs its frame loop under a no-allocation rule (or a memory budget enforced by
// its own allocator), or code running inside a driver callback where allocation is not allowed. For
// them this entry point launches the same frame kernels as arc_trace_frame_dev, but the kernels'
// scratch (the persistent queue head and the GI-ray counter) lives in the file-scope device array
// below instead of context-owned memory. The caller passes the world context (pools uploaded
// earlier) and device pointers for every output, exactly as for arc_trace_frame_dev.
//
// Limits and sharing:
//   - the array is kNoAllocScratchBytes = 256 bytes; every GPU that loads this library holds it
//     until the process exits;
//   - frames are limited to kNoAllocMaxPixels (2^26 = 67,108,864 pixels, e.g. 8192 x 8192): the
//     queue head kept in the array is a 32-bit counter that each warp may push up to 32 entries past
//     the end of the queue, and the limit keeps that far from wrapping; larger frames are rejected
//     with ARC_E_CAPACITY;
//   - every call shares the array: the entry point clears it in stream order before each launch,
//     and calls whose kernels overlap on the GPU (on two streams of one CUDA context) race on it, so
//     callers must not run two of these calls concurrently in one context. Each CUDA context that
//     loads the library holds its own copy of the array;
//   - set-up: the first call in a CUDA context (the context of the arc_ctx's stream, normally the
//     device's primary context) looks up the array's device address with cudaGetSymbolAddress, with
//     that device current, and then makes the caller's previous device current again. The address is
//     kept per device together with the context's unique id, so a context created anew (after
//     cudaDeviceReset, say) is set up again instead of reusing a stale address. Make the first call
//     before any stream capture;
//   - with CUDA's lazy module loading (the default), the first launch of each kernel instance can
//     load its code into device memory. The instance depends on the launch configuration
//     (arc_set_launch_config: variant, register budget) and on whether the frame needs the surface
//     list, so make one warm-up call for each such combination before the region that must not
//     allocate;
//   - a world with water or mirror voxels, or a camera under water, needs the context's surface
//     list (the hits that take those shading branches): reserve it beforehand with
//     arc_reserve_surface_list for at least width x height pixels, else the call fails with
//     ARC_E_CAPACITY.
#include <cuda.h>  // driver API types only: the two driver functions used are fetched through the runtime
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "arc_ctx.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 256;
constexpr uint64_t kNoAllocMaxPixels = 1ull << 26;
constexpr int kMaxDevices = 64;
static_assert(sizeof(arc::Scratch) <= kNoAllocScratchBytes, "frame scratch must fit the static array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
struct ScratchAddr {
    unsigned long long ctx_id = 0;  // unique id of the CUDA context the address belongs to (0 = none yet)
    void* addr = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDevices];

using StreamGetCtxFn = CUresult (*)(CUstream, CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
StreamGetCtxFn g_stream_get_ctx = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int fail(arc_ctx* c, int code, const std::string& msg) {
    c->err = msg;
    return code;
}

// Unique id of the CUDA context the arc_ctx's stream belongs to (the context its kernels run in).
// Call with g_setup_mutex held.
int stream_context_id(arc_ctx* c, unsigned long long* id) {
    if (!g_stream_get_ctx || !g_ctx_get_id) {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuStreamGetCtx", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
            q0 != cudaDriverEntryPointSuccess || !f0 ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || !f1)
            return fail(c, ARC_E_CUDA, "driver entry points cuStreamGetCtx / cuCtxGetId not found");
        g_stream_get_ctx = reinterpret_cast<StreamGetCtxFn>(f0);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    CUcontext ctx = nullptr;
    if (g_stream_get_ctx(reinterpret_cast<CUstream>(c->stream), &ctx) != CUDA_SUCCESS || !ctx ||
        g_ctx_get_id(ctx, id) != CUDA_SUCCESS)
        return fail(c, ARC_E_CUDA, "context of the library stream not found");
    return ARC_OK;
}

// Device address of the static array in the CUDA context of the arc_ctx's stream: looked up once per
// context (set-up), with the arc_ctx's device current, and the caller's current device restored.
int scratch_address(arc_ctx* c, void** out) {
    if (c->device < 0 || c->device >= kMaxDevices) return fail(c, ARC_E_INVALID_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = 0;
    int rc = stream_context_id(c, &id);
    if (rc) return rc;
    ScratchAddr& s = g_scratch_addr[c->device];
    if (s.ctx_id != id || !s.addr) {
        int prev = -1;
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return fail(c, ARC_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        e = cudaSetDevice(c->device);
        if (e != cudaSuccess) return fail(c, ARC_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        const cudaError_t er = prev != c->device ? cudaSetDevice(prev) : cudaSuccess;
        if (e != cudaSuccess || !p)
            return fail(c, ARC_E_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        if (er != cudaSuccess) return fail(c, ARC_E_CUDA, std::string("restoring the current device: ") + cudaGetErrorString(er));
        s.ctx_id = id;
        s.addr = p;
    }
    *out = s.addr;
    return ARC_OK;
}

}  // namespace

extern "C" int arc_trace_frame_noalloc(arc_ctx* c, uint32_t width, uint32_t height, uint32_t* gdm, uint32_t* gnm,
                                       uint32_t* gaa, arc_hit_record* hits, arc_hit_record* gi_hits,
                                       uint64_t* n_gi_dev) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (!gdm || !gnm || !gaa) return fail(c, ARC_E_INVALID_ARG, "null G-buffer");
    if (width == 0 || height == 0) return fail(c, ARC_E_INVALID_ARG, "bad frame size");
    if ((uint64_t)width * height > kNoAllocMaxPixels) {
        char b[200];
        snprintf(b, sizeof b, "frame %ux%u (%llu pixels) exceeds the allocation-free limit of %llu pixels", width, height,
                 (unsigned long long)width * height, (unsigned long long)kNoAllocMaxPixels);
        return fail(c, ARC_E_CAPACITY, b);
    }
    const uint32_t cw = c->cam.world_grid_dims[3] & 0xFFFFu, ch = c->cam.world_grid_dims[3] >> 16;
    if (cw != width || ch != height) return fail(c, ARC_E_INVALID_ARG, "frame size differs from camera world_grid_dims.w");
    void* scratch = nullptr;
    if ((rc = scratch_address(c, &scratch))) return rc;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(arc::Scratch), c->stream);
    if (e != cudaSuccess) return fail(c, ARC_E_CUDA, std::string("clear scratch: ") + cudaGetErrorString(e));
    arc::FrameParams P;
    std::memset(&P, 0, sizeof P);
    P.world = c->world();
    P.width = width;
    P.height = height;
    P.gbuf_depth_mat = gdm;
    P.gbuf_norm_motion = gnm;
    P.gbuf_albedo_ao = gaa;
    P.hits = hits;
    P.gi_hits = gi_hits;
    P.do_gi = 1;
    P.scratch = static_cast<arc::Scratch*>(scratch);
    P.tile_w = c->cfg.tile_w;
    P.tile_h = c->cfg.tile_h;
    P.tiles_x = (width + c->cfg.tile_w - 1u) / c->cfg.tile_w;
    P.queue_len = P.tiles_x * ((height + c->cfg.tile_h - 1u) / c->cfg.tile_h) * 32u;
    P.refill_threshold = c->cfg.refill_threshold;
    P.row0 = 0u;
    P.row_end = height;
    P.gi_mode = arc::kGiRows;
    P.order = c->cfg.order;
    if (c->surface_mats[0] || (c->cam.point_light_count[1] & 0xFFFFu) != 0u) {
        if (c->surf_cap < (size_t)width * height)
            return fail(c, ARC_E_CAPACITY, "surface list not reserved for this frame size (arc_reserve_surface_list)");
        P.surf = c->d_surf;
        P.surf_cap = width * height;
        P.surf_count = &static_cast<arc::Scratch*>(scratch)->surf_count;
    }
    e = arc::launch_frame(P, c->cam, c->cfg, c->n_sm, c->stream);
    if (e != cudaSuccess) return fail(c, ARC_E_CUDA, std::string("frame launch: ") + cudaGetErrorString(e));
    e = arc::launch_surface(P, c->cam, c->n_sm, c->stream);
    if (e != cudaSuccess) return fail(c, ARC_E_CUDA, std::string("surface launch: ") + cudaGetErrorString(e));
    if (n_gi_dev) {
        e = cudaMemcpyAsync(n_gi_dev, &static_cast<arc::Scratch*>(scratch)->gi_rays, sizeof(uint64_t),
                            cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return fail(c, ARC_E_CUDA, std::string("GI count copy: ") + cudaGetErrorString(e));
    }
    return ARC_OK;
}
