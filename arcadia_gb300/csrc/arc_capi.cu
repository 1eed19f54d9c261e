// arc_capi.cu — context, pools and the C ABI of libarc_trace.so.
//
// The context owns the device copies of Arcadia's Group-0 pools (chunk roots, Node64 pool,
// LeafBrick64 pool, 256-entry palette), the camera block, per-launch scratch and a status word
// that device-side range checks write. Host-pointer entry points stage through context-owned device
// buffers; *_dev entry points work on caller device pointers in stream order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "arc_ctx.h"

using arc::Scratch;

namespace {

int set_err(arc_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(arc_ctx* c, cudaError_t e, const char* what) {
    return set_err(c, ARC_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define ARC_CK(ctx, expr)                                          \
    do {                                                           \
        cudaError_t e__ = (expr);                                  \
        if (e__ != cudaSuccess) return cuda_fail((ctx), e__, #expr); \
    } while (0)

inline uint32_t popc64(uint32_t lo, uint32_t hi) { return (uint32_t)__builtin_popcount(lo) + (uint32_t)__builtin_popcount(hi); }

// Range check of a node slice against the pool sizes it will live in.
int validate_nodes(arc_ctx* c, const arc_node64* nodes, uint32_t n, uint32_t node_limit, uint32_t brick_limit, uint32_t first) {
    for (uint32_t i = 0; i < n; ++i) {
        const arc_node64& nd = nodes[i];
        if (nd.mask_low == 0 && nd.mask_high == 0) continue;
        const uint32_t ptr = nd.child_ptr & ARC_PTR_INDEX_MASK;
        if (nd.child_ptr & ARC_IS_LEAF_FLAG) {
            if (!(nd.child_ptr & ARC_IS_UNIFORM_FLAG) && ptr >= brick_limit) {
                char b[160];
                snprintf(b, sizeof b, "node %u: brick index %u >= brick count %u", first + i, ptr, brick_limit);
                return set_err(c, ARC_E_INVALID_POOL, b);
            }
        } else {
            const uint64_t end = (uint64_t)ptr + popc64(nd.mask_low, nd.mask_high);
            if (end > node_limit) {
                char b[160];
                snprintf(b, sizeof b, "node %u: child slice [%u, %llu) beyond node count %u", first + i, ptr,
                         (unsigned long long)end, node_limit);
                return set_err(c, ARC_E_INVALID_POOL, b);
            }
        }
    }
    return ARC_OK;
}

template <typename T>
int ensure_device(arc_ctx* c, T** p, size_t* cap_bytes, size_t need_bytes) {
    if (*cap_bytes >= need_bytes && *p) return ARC_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap_bytes = 0;
    cudaError_t e = cudaMalloc((void**)p, need_bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
    *cap_bytes = need_bytes;
    return ARC_OK;
}

}  // namespace

arc::World arc_ctx::world() const {
    arc::World w;
    w.roots = d_roots;
    w.nodes = reinterpret_cast<const uint4*>(d_nodes);
    w.bricks = reinterpret_cast<const uint32_t*>(d_bricks);
    w.palette = reinterpret_cast<const float4*>(d_palette);
    w.n_nodes = n_nodes;
    w.n_bricks = n_bricks;
    w.n_roots = n_roots;
    w.status = d_status;
    w.bodies = d_bodies;
    w.n_bodies = n_bodies;
    return w;
}

int arc_ctx_check_ready(arc_ctx* c, bool need_cam) {
    if (!c) return ARC_E_INVALID_ARG;
    if (!c->have_world) return set_err(c, ARC_E_NO_WORLD, "no world uploaded");
    if (need_cam && !c->have_cam) return set_err(c, ARC_E_NO_CAMERA, "no camera set");
    return ARC_OK;
}

int arc_ctx_finish(arc_ctx* c) {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamSynchronize");
    if (c->timing_pending) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->last_ms = ms;
        c->timing_pending = false;
    }
    uint32_t st = 0;
    e = cudaMemcpy(&st, c->d_status, sizeof st, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "status readback");
    c->last_status = st;
    if (st) {
        char b[128];
        snprintf(b, sizeof b, (st & 0x80000000u) ? "tensor-core pipeline wait timed out (status 0x%x)"
                                                 : "device range check failed (status 0x%x): pool index out of range",
                 st);
        cudaMemsetAsync(c->d_status, 0, sizeof(uint32_t), c->stream);
        cudaStreamSynchronize(c->stream);
        return set_err(c, ARC_E_DEVICE_CHECK, b);
    }
    return ARC_OK;
}

// Device table of World records: slot 0 = the context's main world, slots 1.. = arc_upload_world_slot.
int arc_ctx_sync_world_table(arc_ctx* c) {
    if (!c->d_worlds) {
        cudaError_t e = cudaMalloc((void**)&c->d_worlds, sizeof(arc::World) * arc_ctx::kSlots);
        if (e != cudaSuccess) return cuda_fail(c, e, "world table");
    }
    arc::World tab[arc_ctx::kSlots];
    memset(tab, 0, sizeof tab);
    tab[0] = c->world();
    for (int i = 1; i < arc_ctx::kSlots; ++i) {
        const arc_ctx::Slot& sl = c->slots[i];
        if (!sl.valid) continue;
        tab[i].roots = sl.d_roots;
        tab[i].nodes = reinterpret_cast<const uint4*>(sl.d_nodes);
        tab[i].bricks = reinterpret_cast<const uint32_t*>(sl.d_bricks);
        tab[i].palette = reinterpret_cast<const float4*>(sl.d_palette);
        tab[i].n_nodes = sl.n_nodes;
        tab[i].n_bricks = sl.n_bricks;
        tab[i].n_roots = sl.n_roots;
        tab[i].status = c->d_status;
    }
    cudaError_t e = cudaMemcpyAsync(c->d_worlds, tab, sizeof tab, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "world table upload");
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "world table upload");
    return ARC_OK;
}

int arc_ctx_stage(arc_ctx* c, size_t bytes, void** out) {
    int rc = ensure_device(c, reinterpret_cast<unsigned char**>(&c->d_stage), &c->stage_bytes, bytes);
    if (rc) return rc;
    *out = c->d_stage;
    return ARC_OK;
}

int arc_ctx_side_begin(arc_ctx* c) {
    if (!c->side_stream) {
        ARC_CK(c, cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking));
        ARC_CK(c, cudaEventCreateWithFlags(&c->side_fork, cudaEventDisableTiming));
        ARC_CK(c, cudaEventCreateWithFlags(&c->side_join, cudaEventDisableTiming));
    }
    ARC_CK(c, cudaEventRecord(c->side_fork, c->stream));
    ARC_CK(c, cudaStreamWaitEvent(c->side_stream, c->side_fork, 0));
    std::swap(c->stream, c->side_stream);
    return ARC_OK;
}

int arc_ctx_side_end(arc_ctx* c) {
    std::swap(c->stream, c->side_stream);
    ARC_CK(c, cudaEventRecord(c->side_join, c->side_stream));
    return ARC_OK;
}

int arc_ctx_side_join(arc_ctx* c) {
    ARC_CK(c, cudaStreamWaitEvent(c->stream, c->side_join, 0));
    return ARC_OK;
}

int arc_ctx_reserve_surface(arc_ctx* c, size_t entries) {
    if (c->surf_cap >= entries && c->d_surf_count) return ARC_OK;
    ARC_CK(c, cudaStreamSynchronize(c->stream));
    if (c->copy_stream)
        for (int i = 0; i < arc_ctx::kMaxBands; ++i) ARC_CK(c, cudaStreamSynchronize(c->band_stream[i]));
    cudaFree(c->d_surf);
    c->d_surf = nullptr;
    c->surf_cap = 0;
    if (!c->d_surf_count) ARC_CK(c, cudaMalloc((void**)&c->d_surf_count, sizeof(uint32_t) * arc_ctx::kMaxBands));
    ARC_CK(c, cudaMalloc((void**)&c->d_surf, sizeof(arc::SurfaceEntry) * std::max<size_t>(entries, 1)));
    c->surf_cap = entries;
    return ARC_OK;
}

bool arc_pools_have_surface_mats(const arc_node64* nodes, uint32_t n_nodes, const arc_brick64* bricks, uint32_t n_bricks) {
    for (uint32_t i = 0; i < n_nodes; ++i) {
        const uint32_t m = nodes[i].lod_payload >> 24;
        if (m == arc::kMatWaterCrystal || m == arc::kMatMirrorChrome) return true;
    }
    // a zero byte in w ^ 0x12121212 (0x1C1C1C1C) is a material-18 (28) voxel
    auto has_zero_byte = [](uint32_t v) { return ((v - 0x01010101u) & ~v & 0x80808080u) != 0u; };
    for (uint32_t i = 0; i < n_bricks; ++i)
        for (uint32_t w : bricks[i].packed_materials)
            if (has_zero_byte(w ^ 0x12121212u) || has_zero_byte(w ^ 0x1C1C1C1Cu)) return true;
    return false;
}

extern "C" {

int arc_create(int device, arc_ctx** out) {
    if (!out) return ARC_E_INVALID_ARG;
    *out = nullptr;
    arc_ctx* c = new (std::nothrow) arc_ctx();
    if (!c) return ARC_E_OUT_OF_MEMORY;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { int rc = cuda_fail(c, e, "cudaSetDevice"); delete c; return rc; }
    cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device);
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc((void**)&c->d_scratch, sizeof(Scratch))) != cudaSuccess ||
        (e = cudaMalloc((void**)&c->d_status, sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
        int rc = cuda_fail(c, e, "context setup");
        arc_destroy(c);
        return rc;
    }
    cudaMemset(c->d_scratch, 0, sizeof(Scratch));
    cudaMemset(c->d_status, 0, sizeof(uint32_t));
    // the plain kernel with the GI rays as their own pass (the autotuner's pick on the 1080p caves frame)
    c->cfg.variant = 0;
    c->cfg.block_threads = 128;
    c->cfg.blocks_per_sm = 0;
    c->cfg.tile_w = 8;
    c->cfg.tile_h = 4;
    c->cfg.refill_threshold = 24;
    c->cfg.reg_blocks = 3;
    c->cfg.order = 1;  // Morton block order: 2 % faster than row-major on the 1080p caves frame
    c->cfg.features = 0;
    *out = c;
    return ARC_OK;
}

int arc_destroy(arc_ctx* c) {
    if (!c) return ARC_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->d_roots);
    cudaFree(c->d_nodes);
    cudaFree(c->d_bricks);
    cudaFree(c->d_palette);
    cudaFree(c->d_scratch);
    cudaFree(c->d_status);
    cudaFree(c->d_stage);
    cudaFree(c->d_gisort);
    cudaFree(c->d_top);
    cudaFree(c->d_sharc_keys);
    cudaFree(c->d_sharc_accum);
    cudaFree(c->d_sharc_resolved);
    cudaFree(c->d_sharc_stage);
    for (int i = 1; i < arc_ctx::kSlots; ++i) {
        cudaFree(c->slots[i].d_roots);
        cudaFree(c->slots[i].d_nodes);
        cudaFree(c->slots[i].d_bricks);
        cudaFree(c->slots[i].d_palette);
    }
    cudaFree(c->d_worlds);
    cudaFree(c->d_views);
    if (c->h_views) cudaFreeHost(c->h_views);
    if (c->views_exec) cudaGraphExecDestroy(c->views_exec);
    if (c->views_graph) cudaGraphDestroy(c->views_graph);
    cudaFree(c->d_nrc_w32);
    cudaFree(c->d_nrc_w16);
    cudaFree(c->d_nrc_w16_ema);
    cudaFree(c->d_nrc_wu_ema);
    cudaFree(c->d_nrc_wu);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
        cudaStreamSynchronize(c->gi_copy_stream);
        cudaStreamDestroy(c->gi_copy_stream);
        for (int i = 0; i < arc_ctx::kMaxBands; ++i) {
            cudaStreamSynchronize(c->band_stream[i]);
            cudaStreamDestroy(c->band_stream[i]);
            cudaEventDestroy(c->band_ev[i]);
            cudaEventDestroy(c->band_gev[i]);
        }
        cudaEventDestroy(c->copies_done);
        cudaEventDestroy(c->gi_copies_done);
        cudaEventDestroy(c->frame_start);
    }
    cudaFree(c->d_surf);
    cudaFree(c->d_surf_count);
    cudaFree(c->d_bodies);
    cudaFree(c->d_edit);
    cudaFree(c->d_edit_stage);
    cudaFreeHost(c->h_edit_stage);
    cudaFree(c->d_nrc_batch);
    cudaFree(c->d_nrc_gate);
    cudaFree(c->d_nrc_loss);
    if (c->side_stream) {
        cudaStreamSynchronize(c->side_stream);
        cudaStreamDestroy(c->side_stream);
        cudaEventDestroy(c->side_fork);
        cudaEventDestroy(c->side_join);
    }
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return ARC_OK;
}

int arc_last_error(const arc_ctx* c, char* buf, size_t n) {
    if (!c || !buf || n == 0) return ARC_E_INVALID_ARG;
    snprintf(buf, n, "%s", c->err.c_str());
    return ARC_OK;
}

int arc_synchronize(arc_ctx* c) {
    if (!c) return ARC_E_INVALID_ARG;
    return arc_ctx_finish(c);
}

int arc_get_stream(arc_ctx* c, void** stream) {
    if (!c || !stream) return ARC_E_INVALID_ARG;
    *stream = (void*)c->stream;
    return ARC_OK;
}

int arc_debug_set(arc_ctx* c, int what, long long value) {
    if (!c) return ARC_E_INVALID_ARG;
    switch (what) {
        case ARC_DEBUG_TC_WAIT_BUDGET:
            if (value < 0) return set_err(c, ARC_E_INVALID_ARG, "wait budget must be >= 0 cycles");
            c->tc_wait_budget = value;
            return ARC_OK;
        case ARC_DEBUG_TC_STALL:
            c->tc_stall = value != 0;
            return ARC_OK;
        case ARC_DEBUG_SKIP_POOL_VALIDATION:
            c->skip_pool_validation = value != 0;
            return ARC_OK;
        default:
            return set_err(c, ARC_E_INVALID_ARG, "unknown debug hook");
    }
}

int arc_set_launch_config(arc_ctx* c, const arc_launch_config* cfg) {
    if (!c || !cfg) return ARC_E_INVALID_ARG;
    if (cfg->variant > 1u) return set_err(c, ARC_E_INVALID_ARG, "variant must be 0 or 1");
    if (cfg->block_threads == 0 || cfg->block_threads % 32u)
        return set_err(c, ARC_E_INVALID_ARG, "block_threads must be a multiple of 32");
    if (cfg->variant == 0u && cfg->block_threads % 8u) return set_err(c, ARC_E_INVALID_ARG, "plain variant needs block_threads % 8 == 0");
    if (cfg->tile_w * cfg->tile_h != 32u) return set_err(c, ARC_E_INVALID_ARG, "tile_w * tile_h must be 32");
    if (cfg->refill_threshold < 1u || cfg->refill_threshold > 32u) return set_err(c, ARC_E_INVALID_ARG, "refill_threshold in [1, 32]");
    if (cfg->block_threads > 256u) return set_err(c, ARC_E_INVALID_ARG, "block_threads <= 256");
    if (cfg->reg_blocks < 1u || cfg->reg_blocks > 4u) return set_err(c, ARC_E_INVALID_ARG, "reg_blocks in [1, 4]");
    if (cfg->order > 1u) return set_err(c, ARC_E_INVALID_ARG, "order must be 0 (row-major) or 1 (Morton)");
    if (cfg->features & ~(ARC_FEAT_WARP_FETCH | ARC_FEAT_NODE_VISIT | ARC_FEAT_GI_SORT | ARC_FEAT_TOP_TABLE | ARC_FEAT_GRID_STRIDE |
                          ARC_FEAT_PRECOMP | ARC_FEAT_GI_REPACK))
        return set_err(c, ARC_E_INVALID_ARG, "unknown feature bits");
    c->cfg = *cfg;
    return ARC_OK;
}

int arc_set_frame_bands(arc_ctx* c, uint32_t n) {
    if (!c) return ARC_E_INVALID_ARG;
    if (n > (uint32_t)arc_ctx::kMaxBands) return set_err(c, ARC_E_INVALID_ARG, "frame bands in [0, 8]");
    c->frame_bands = n;
    return ARC_OK;
}

int arc_get_launch_config(const arc_ctx* c, arc_launch_config* cfg) {
    if (!c || !cfg) return ARC_E_INVALID_ARG;
    *cfg = c->cfg;
    return ARC_OK;
}

int arc_get_stats(const arc_ctx* c, arc_stats* out) {
    if (!c || !out) return ARC_E_INVALID_ARG;
    out->last_kernel_ms = c->last_ms;
    out->rays_traced = c->last_rays;
    out->device_status = c->last_status;
    out->n_sm = (uint32_t)c->n_sm;
    return ARC_OK;
}

int arc_upload_world(arc_ctx* c, const uint32_t grid[3], const uint32_t* roots, uint32_t n_roots, const arc_node64* nodes,
                     uint32_t n_nodes, const arc_brick64* bricks, uint32_t n_bricks, const arc_material* palette,
                     uint32_t node_headroom, uint32_t brick_headroom) {
    if (!c || !grid || !roots || !nodes || !palette || n_nodes == 0) return set_err(c, ARC_E_INVALID_ARG, "null pool or empty node pool");
    if (n_bricks && !bricks) return set_err(c, ARC_E_INVALID_ARG, "null brick pool");
    for (int i = 0; i < 3; ++i)
        if (grid[i] == 0 || grid[i] > 1024u) return set_err(c, ARC_E_INVALID_ARG, "grid dims must be in [1, 1024]");
    const uint64_t nch = (uint64_t)grid[0] * grid[1] * grid[2];
    if (nch != n_roots) return set_err(c, ARC_E_INVALID_ARG, "n_roots != grid volume");
    const uint64_t cap_nodes = (uint64_t)n_nodes + node_headroom, cap_bricks = (uint64_t)std::max<uint32_t>(n_bricks, 1u) + brick_headroom;
    if (cap_nodes > ARC_PTR_INDEX_MASK || cap_bricks > ARC_PTR_INDEX_MASK) return set_err(c, ARC_E_CAPACITY, "pool beyond 30-bit index range");
    int rc = ARC_OK;
    if (!c->skip_pool_validation) {  // only a test's fault injection turns this off (arc_debug_set)
        for (uint32_t i = 0; i < n_roots; ++i)
            if (roots[i] != ARC_EMPTY_CHUNK && roots[i] >= n_nodes) {
                char b[128];
                snprintf(b, sizeof b, "chunk %u: root %u >= node count %u", i, roots[i], n_nodes);
                return set_err(c, ARC_E_INVALID_POOL, b);
            }
        if ((rc = validate_nodes(c, nodes, n_nodes, n_nodes, n_bricks, 0))) return rc;
    }
    ARC_CK(c, cudaSetDevice(c->device));
    ARC_CK(c, cudaStreamSynchronize(c->stream));
    cudaFree(c->d_roots);
    cudaFree(c->d_nodes);
    cudaFree(c->d_bricks);
    c->d_roots = nullptr;
    c->d_nodes = nullptr;
    c->d_bricks = nullptr;
    c->have_world = false;
    ARC_CK(c, cudaMalloc((void**)&c->d_roots, sizeof(uint32_t) * n_roots));
    ARC_CK(c, cudaMalloc((void**)&c->d_nodes, sizeof(arc_node64) * cap_nodes));
    ARC_CK(c, cudaMalloc((void**)&c->d_bricks, sizeof(arc_brick64) * cap_bricks));
    if (!c->d_palette) ARC_CK(c, cudaMalloc((void**)&c->d_palette, sizeof(arc_material) * 256));
    ARC_CK(c, cudaMemcpyAsync(c->d_roots, roots, sizeof(uint32_t) * n_roots, cudaMemcpyHostToDevice, c->stream));
    ARC_CK(c, cudaMemcpyAsync(c->d_nodes, nodes, sizeof(arc_node64) * n_nodes, cudaMemcpyHostToDevice, c->stream));
    if (n_bricks) ARC_CK(c, cudaMemcpyAsync(c->d_bricks, bricks, sizeof(arc_brick64) * n_bricks, cudaMemcpyHostToDevice, c->stream));
    else ARC_CK(c, cudaMemsetAsync(c->d_bricks, 0, sizeof(arc_brick64), c->stream));
    // headroom starts empty: growth from patches or in-place edits lands here
    if (cap_nodes > n_nodes)
        ARC_CK(c, cudaMemsetAsync(c->d_nodes + n_nodes, 0, sizeof(arc_node64) * (cap_nodes - n_nodes), c->stream));
    const uint32_t nb0 = std::max<uint32_t>(n_bricks, 1u);
    if (cap_bricks > nb0)
        ARC_CK(c, cudaMemsetAsync(c->d_bricks + nb0, 0, sizeof(arc_brick64) * (cap_bricks - nb0), c->stream));
    ARC_CK(c, cudaMemcpyAsync(c->d_palette, palette, sizeof(arc_material) * 256, cudaMemcpyHostToDevice, c->stream));
    ARC_CK(c, cudaStreamSynchronize(c->stream));
    c->grid[0] = grid[0];
    c->grid[1] = grid[1];
    c->grid[2] = grid[2];
    c->n_roots = n_roots;
    c->n_nodes = n_nodes;
    c->cap_nodes = (uint32_t)cap_nodes;
    c->n_bricks = std::max<uint32_t>(n_bricks, 1u);
    c->cap_bricks = (uint32_t)cap_bricks;
    c->have_world = true;
    c->surface_mats[0] = arc_pools_have_surface_mats(nodes, n_nodes, bricks, n_bricks);
    if ((rc = arc_edit_reset(c))) return rc;
    return arc_ctx_sync_world_table(c);
}

int arc_upload_world_slot(arc_ctx* c, uint32_t slot, const uint32_t grid[3], const uint32_t* roots, uint32_t n_roots,
                          const arc_node64* nodes, uint32_t n_nodes, const arc_brick64* bricks, uint32_t n_bricks,
                          const arc_material* palette) {
    if (!c) return ARC_E_INVALID_ARG;
    if (slot == 0) return arc_upload_world(c, grid, roots, n_roots, nodes, n_nodes, bricks, n_bricks, palette, 0, 0);
    if (slot >= (uint32_t)arc_ctx::kSlots) return set_err(c, ARC_E_INVALID_ARG, "world slot out of range");
    if (!grid || !roots || !nodes || !palette || n_nodes == 0) return set_err(c, ARC_E_INVALID_ARG, "null pool");
    if (n_bricks && !bricks) return set_err(c, ARC_E_INVALID_ARG, "null brick pool");
    for (int i = 0; i < 3; ++i)
        if (grid[i] == 0 || grid[i] > 1024u) return set_err(c, ARC_E_INVALID_ARG, "grid dims must be in [1, 1024]");
    if ((uint64_t)grid[0] * grid[1] * grid[2] != n_roots) return set_err(c, ARC_E_INVALID_ARG, "n_roots != grid volume");
    for (uint32_t i = 0; i < n_roots; ++i)
        if (roots[i] != ARC_EMPTY_CHUNK && roots[i] >= n_nodes) return set_err(c, ARC_E_INVALID_POOL, "root out of range");
    int rc = validate_nodes(c, nodes, n_nodes, n_nodes, n_bricks, 0);
    if (rc) return rc;
    ARC_CK(c, cudaStreamSynchronize(c->stream));
    arc_ctx::Slot& sl = c->slots[slot];
    cudaFree(sl.d_roots);
    cudaFree(sl.d_nodes);
    cudaFree(sl.d_bricks);
    sl = arc_ctx::Slot();
    const uint32_t nb = std::max<uint32_t>(n_bricks, 1u);
    ARC_CK(c, cudaMalloc((void**)&sl.d_roots, sizeof(uint32_t) * n_roots));
    ARC_CK(c, cudaMalloc((void**)&sl.d_nodes, sizeof(arc_node64) * n_nodes));
    ARC_CK(c, cudaMalloc((void**)&sl.d_bricks, sizeof(arc_brick64) * nb));
    ARC_CK(c, cudaMalloc((void**)&sl.d_palette, sizeof(arc_material) * 256));
    ARC_CK(c, cudaMemcpyAsync(sl.d_roots, roots, sizeof(uint32_t) * n_roots, cudaMemcpyHostToDevice, c->stream));
    ARC_CK(c, cudaMemcpyAsync(sl.d_nodes, nodes, sizeof(arc_node64) * n_nodes, cudaMemcpyHostToDevice, c->stream));
    if (n_bricks) ARC_CK(c, cudaMemcpyAsync(sl.d_bricks, bricks, sizeof(arc_brick64) * n_bricks, cudaMemcpyHostToDevice, c->stream));
    else ARC_CK(c, cudaMemsetAsync(sl.d_bricks, 0, sizeof(arc_brick64), c->stream));
    ARC_CK(c, cudaMemcpyAsync(sl.d_palette, palette, sizeof(arc_material) * 256, cudaMemcpyHostToDevice, c->stream));
    sl.grid[0] = grid[0];
    sl.grid[1] = grid[1];
    sl.grid[2] = grid[2];
    sl.n_roots = n_roots;
    sl.n_nodes = n_nodes;
    sl.n_bricks = nb;
    sl.valid = true;
    c->surface_mats[slot] = arc_pools_have_surface_mats(nodes, n_nodes, bricks, n_bricks);
    return arc_ctx_sync_world_table(c);
}

int arc_apply_patch(arc_ctx* c, uint32_t chunk, uint32_t new_root, uint32_t node_offset, const arc_node64* nodes,
                    uint32_t n_nodes, uint32_t brick_offset, const arc_brick64* bricks, uint32_t n_bricks) {
    int rc = arc_ctx_check_ready(c, false);
    if (rc) return rc;
    if (chunk >= c->n_roots) return set_err(c, ARC_E_INVALID_ARG, "chunk index out of range");
    if ((n_nodes && !nodes) || (n_bricks && !bricks)) return set_err(c, ARC_E_INVALID_ARG, "null patch slice");
    if ((uint64_t)node_offset + n_nodes > c->cap_nodes || (uint64_t)brick_offset + n_bricks > c->cap_bricks)
        return set_err(c, ARC_E_CAPACITY, "patch beyond pool capacity (re-upload with more headroom)");
    const uint32_t node_limit = std::max<uint32_t>(c->n_nodes, node_offset + n_nodes);
    const uint32_t brick_limit = std::max<uint32_t>(c->n_bricks, brick_offset + n_bricks);
    if (new_root != ARC_EMPTY_CHUNK && new_root >= node_limit) return set_err(c, ARC_E_INVALID_POOL, "patch root out of range");
    rc = validate_nodes(c, nodes, n_nodes, node_limit, brick_limit, node_offset);
    if (rc) return rc;
    if (n_nodes) ARC_CK(c, cudaMemcpyAsync(c->d_nodes + node_offset, nodes, sizeof(arc_node64) * n_nodes, cudaMemcpyHostToDevice, c->stream));
    if (n_bricks) ARC_CK(c, cudaMemcpyAsync(c->d_bricks + brick_offset, bricks, sizeof(arc_brick64) * n_bricks, cudaMemcpyHostToDevice, c->stream));
    ARC_CK(c, cudaMemcpyAsync(c->d_roots + chunk, &new_root, sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
    if ((rc = arc_edit_raise_floor(c, node_offset + n_nodes, brick_offset + n_bricks))) return rc;
    ARC_CK(c, cudaStreamSynchronize(c->stream));
    c->n_nodes = node_limit;
    c->n_bricks = brick_limit;
    if (arc_pools_have_surface_mats(nodes, n_nodes, bricks, n_bricks)) c->surface_mats[0] = true;
    return arc_ctx_sync_world_table(c);
}

int arc_reserve_surface_list(arc_ctx* c, uint64_t max_pixels) {
    if (!c) return ARC_E_INVALID_ARG;
    if (max_pixels == 0 || max_pixels > (1ull << 32)) return set_err(c, ARC_E_INVALID_ARG, "max_pixels must be in [1, 2^32]");
    ARC_CK(c, cudaSetDevice(c->device));
    return arc_ctx_reserve_surface(c, (size_t)max_pixels);
}

int arc_set_camera(arc_ctx* c, const arc_camera_uniforms* cam) {
    if (!c || !cam) return ARC_E_INVALID_ARG;
    const uint32_t w = cam->world_grid_dims[3] & 0xFFFFu, h = cam->world_grid_dims[3] >> 16;
    if (c->have_world && (cam->world_grid_dims[0] != c->grid[0] || cam->world_grid_dims[1] != c->grid[1] ||
                          cam->world_grid_dims[2] != c->grid[2]))
        return set_err(c, ARC_E_INVALID_ARG, "camera world_grid_dims do not match the uploaded world");
    (void)w;
    (void)h;
    c->cam = *cam;
    c->have_cam = true;
    return ARC_OK;
}

// ------------------------------------------------------------------------------------------------
// Frame passes
// ------------------------------------------------------------------------------------------------

static int check_dims(arc_ctx* c, uint32_t width, uint32_t height) {
    if (width == 0 || height == 0 || width > 0xFFFFu || height > 0xFFFFu) return set_err(c, ARC_E_INVALID_ARG, "bad frame size");
    const uint32_t w = c->cam.world_grid_dims[3] & 0xFFFFu, h = c->cam.world_grid_dims[3] >> 16;
    if (w != width || h != height) return set_err(c, ARC_E_INVALID_ARG, "frame size differs from camera world_grid_dims.w");
    return ARC_OK;
}

// Restricts a frame launch to rows [row0, row_end) (the persistent kernel's queue covers those rows).
static void frame_rows(arc_ctx* c, arc::FrameParams& P, uint32_t row0, uint32_t row_end) {
    P.row0 = row0;
    P.row_end = row_end;
    const uint32_t tiles_y = (row_end - row0 + c->cfg.tile_h - 1u) / c->cfg.tile_h;
    P.queue_len = P.tiles_x * tiles_y * 32u;
}

static arc::FrameParams frame_params(arc_ctx* c, uint32_t width, uint32_t height) {
    arc::FrameParams P;
    memset(&P, 0, sizeof P);
    P.world = c->world();
    P.width = width;
    P.height = height;
    P.scratch = c->d_scratch;
    P.tile_w = c->cfg.tile_w;
    P.tile_h = c->cfg.tile_h;
    P.tiles_x = (width + c->cfg.tile_w - 1u) / c->cfg.tile_w;
    P.refill_threshold = c->cfg.refill_threshold;
    P.gi_mode = arc::kGiRows;  // honoured by the plain kernel; the persistent kernel fuses the GI ray
    P.order = c->cfg.order;
    if (c->cfg.variant == 0u && (c->cfg.features & (ARC_FEAT_TOP_TABLE | ARC_FEAT_GRID_STRIDE))) {
        if (!c->d_top && cudaMalloc((void**)&c->d_top, sizeof(uint4) * arc::kTopMaxNodes + 16u) != cudaSuccess)
            c->d_top = nullptr;  // without the table the plain kernel runs
        if (c->d_top) {
            P.top = reinterpret_cast<uint4*>(c->d_top);
            P.top_info = reinterpret_cast<uint32_t*>(c->d_top + sizeof(uint4) * arc::kTopMaxNodes);
        }
    }
    frame_rows(c, P, 0u, height);
    return P;
}

static bool cam_underwater(const arc_camera_uniforms& cam) { return (cam.point_light_count[1] & 0xFFFFu) != 0u; }

// Surface list for the rows of P (the listed hits are shaded after the frame kernel): none when the
// world holds no water or mirror voxel and the camera is above water. `count` is a counter that is
// zero when the launch starts.
static int surface_prepare(arc_ctx* c, arc::FrameParams& P, uint32_t* count) {
    P.surf = nullptr;
    P.surf_count = nullptr;
    P.surf_cap = 0;
    if (!c->surface_mats[0] && !cam_underwater(c->cam)) return ARC_OK;
    int rc = arc_ctx_reserve_surface(c, (size_t)P.width * P.height);
    if (rc) return rc;
    P.surf = c->d_surf + (size_t)P.row0 * P.width;
    P.surf_cap = (P.row_end - P.row0) * P.width;
    P.surf_count = count;
    return ARC_OK;
}

static int ensure_band_streams(arc_ctx* c);

// Bands of a device frame: the plain kernel's launches over the whole frame, or (frame_bands > 1)
// over horizontal bands on the band streams, forked from and joined back to the context stream, so
// that one band's GI pass runs in another band's primary-kernel tail. The variants with frame-wide
// scratch (the GI rays sorted over the frame, the resident-CTA primary with its staged table), the
// persistent kernel (one queue) and primary-only frames (no GI pass to fill the tails: 0.479 against
// 0.464 ms at 1080p in four bands) keep one launch. Every pixel is computed by the same code either way.
static uint32_t device_bands(const arc_ctx* c, const arc::FrameParams& P) {
    if (c->cfg.variant != 0u || !P.do_gi ||
        (c->cfg.features & (ARC_FEAT_GI_SORT | ARC_FEAT_TOP_TABLE | ARC_FEAT_GRID_STRIDE)))
        return 1u;
    const uint32_t want = c->frame_bands ? c->frame_bands : arc_ctx::kDefaultFrameBands;
    return std::max<uint32_t>(1u, std::min<uint32_t>(want, (P.row_end - P.row0) / 64u));
}

// First row of band b of n: equal bands, edges on multiples of 32 rows (whole blocks of every kernel).
static uint32_t device_band_edge(uint32_t row0, uint32_t row_end, uint32_t b, uint32_t n) {
    if (b >= n) return row_end;
    return row0 + (uint32_t)(((uint64_t)(row_end - row0) * b / n) & ~(uint64_t)31);
}

static int run_frame(arc_ctx* c, arc::FrameParams& P) {
    const uint32_t nb = device_bands(c, P);
    if (nb > 1u) {
        int rc = ensure_band_streams(c);
        if (rc) return rc;
        const bool surf = c->surface_mats[0] || cam_underwater(c->cam);
        ARC_CK(c, cudaMemsetAsync(c->d_scratch, 0, sizeof(Scratch), c->stream));
        if (surf) {
            if ((rc = arc_ctx_reserve_surface(c, (size_t)P.width * P.height))) return rc;
            ARC_CK(c, cudaMemsetAsync(c->d_surf_count, 0, sizeof(uint32_t) * arc_ctx::kMaxBands, c->stream));
        }
        ARC_CK(c, cudaEventRecord(c->ev0, c->stream));
        ARC_CK(c, cudaEventRecord(c->frame_start, c->stream));
        const uint32_t r0 = P.row0, r1 = P.row_end;
        for (uint32_t b = 0; b < nb; ++b) {
            arc::FrameParams Pb = P;
            frame_rows(c, Pb, device_band_edge(r0, r1, b, nb), device_band_edge(r0, r1, b + 1u, nb));
            cudaStream_t st = c->band_stream[b];
            ARC_CK(c, cudaStreamWaitEvent(st, c->frame_start, 0));
            if ((rc = surface_prepare(c, Pb, c->d_surf_count + b))) return rc;
            ARC_CK(c, arc::launch_frame(Pb, c->cam, c->cfg, c->n_sm, st));
            ARC_CK(c, arc::launch_surface(Pb, c->cam, c->n_sm, st));
            ARC_CK(c, cudaEventRecord(c->band_ev[b], st));
        }
        for (uint32_t b = 0; b < nb; ++b) ARC_CK(c, cudaStreamWaitEvent(c->stream, c->band_ev[b], 0));
        ARC_CK(c, cudaEventRecord(c->ev1, c->stream));
        c->timing_pending = true;
        return ARC_OK;
    }
    int rc = surface_prepare(c, P, &c->d_scratch->surf_count);
    if (rc) return rc;
    ARC_CK(c, cudaMemsetAsync(c->d_scratch, 0, sizeof(Scratch), c->stream));
    ARC_CK(c, cudaEventRecord(c->ev0, c->stream));
    ARC_CK(c, arc::launch_frame(P, c->cam, c->cfg, c->n_sm, c->stream));
    ARC_CK(c, arc::launch_surface(P, c->cam, c->n_sm, c->stream));
    ARC_CK(c, cudaEventRecord(c->ev1, c->stream));
    c->timing_pending = true;
    return ARC_OK;
}

static int collect_frame(arc_ctx* c, uint64_t primary_rays, uint64_t* n_gi_host) {
    Scratch s;
    ARC_CK(c, cudaMemcpyAsync(&s, c->d_scratch, sizeof s, cudaMemcpyDeviceToHost, c->stream));
    int rc = arc_ctx_finish(c);
    if (rc) return rc;
    float ms = 0.0f;
    if (c->timing_pending && cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->last_ms = ms;
    c->timing_pending = false;
    c->last_rays = primary_rays + s.gi_rays;
    if (n_gi_host) *n_gi_host = s.gi_rays;
    return ARC_OK;
}

int arc_trace_frame_dev(arc_ctx* c, uint32_t width, uint32_t height, uint32_t* gdm, uint32_t* gnm, uint32_t* gaa,
                        arc_hit_record* hits, arc_hit_record* gi_hits, uint64_t* n_gi_dev) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if ((rc = check_dims(c, width, height))) return rc;
    if (!gdm || !gnm || !gaa) return set_err(c, ARC_E_INVALID_ARG, "null G-buffer");
    arc::FrameParams P = frame_params(c, width, height);
    P.gbuf_depth_mat = gdm;
    P.gbuf_norm_motion = gnm;
    P.gbuf_albedo_ao = gaa;
    P.hits = hits;
    P.gi_hits = gi_hits;
    P.do_gi = 1;
    if (c->cfg.variant == 0u && (c->cfg.features & ARC_FEAT_GI_SORT)) {
        // scratch of the globally sorted GI pass: bins (+ total), per-pixel ray and key, sorted rays
        const size_t npx = (size_t)width * height, bins_bytes = 256u * ((sizeof(uint32_t) * (arc::kGiSortBins + 1u) + 255u) / 256u);
        if ((rc = ensure_device(c, &c->d_gisort, &c->gisort_bytes, bins_bytes + 64u * npx))) return rc;
        P.gisort.bins = reinterpret_cast<uint32_t*>(c->d_gisort);
        P.gisort.ray_pix = reinterpret_cast<float4*>(c->d_gisort + bins_bytes);
        P.gisort.ray_dir = P.gisort.ray_pix + npx;
        P.gisort.sorted = P.gisort.ray_dir + npx;
        const uint32_t ext = std::max(c->grid[0], std::max(c->grid[1], c->grid[2])) * 256u;
        uint32_t sh = 0u;
        while (((ext - 1u) >> sh) >= 16u) ++sh;
        P.gisort.cell_shift = sh;
    }
    if ((rc = run_frame(c, P))) return rc;
    if (n_gi_dev) ARC_CK(c, cudaMemcpyAsync(n_gi_dev, &c->d_scratch->gi_rays, sizeof(uint64_t), cudaMemcpyDeviceToDevice, c->stream));
    c->last_rays = (uint64_t)width * height;
    return ARC_OK;
}

int arc_trace_primary_dev(arc_ctx* c, uint32_t width, uint32_t height, uint32_t* gdm, uint32_t* gnm, uint32_t* gaa,
                          arc_hit_record* hits) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if ((rc = check_dims(c, width, height))) return rc;
    if (!gdm || !gnm || !gaa) return set_err(c, ARC_E_INVALID_ARG, "null G-buffer");
    arc::FrameParams P = frame_params(c, width, height);
    P.gbuf_depth_mat = gdm;
    P.gbuf_norm_motion = gnm;
    P.gbuf_albedo_ao = gaa;
    P.hits = hits;
    P.do_gi = 0;
    return run_frame(c, P);
}

int arc_trace_secondary_dev(arc_ctx* c, uint32_t width, uint32_t height, const uint32_t* gdm, const uint32_t* gnm,
                            arc_hit_record* gi_hits) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if ((rc = check_dims(c, width, height))) return rc;
    if (!gdm || !gnm || !gi_hits) return set_err(c, ARC_E_INVALID_ARG, "null buffer");
    arc::FrameParams P = frame_params(c, width, height);
    P.gbuf_depth_mat = const_cast<uint32_t*>(gdm);
    P.gbuf_norm_motion = const_cast<uint32_t*>(gnm);
    P.gi_hits = gi_hits;
    // the GI pass counts its rays into the context scratch; start that count at zero as a frame does
    ARC_CK(c, cudaMemsetAsync(c->d_scratch, 0, sizeof(arc::Scratch), c->stream));
    ARC_CK(c, arc::launch_secondary(P, c->cam, c->cfg, c->stream));
    return ARC_OK;
}

// Host-buffer variants: stage outputs in one context-owned device block.
static int ensure_band_streams(arc_ctx* c) {
    if (c->copy_stream) return ARC_OK;
    ARC_CK(c, cudaStreamCreateWithFlags(&c->gi_copy_stream, cudaStreamNonBlocking));
    ARC_CK(c, cudaEventCreateWithFlags(&c->gi_copies_done, cudaEventDisableTiming));
    for (int i = 0; i < arc_ctx::kMaxBands; ++i)
        ARC_CK(c, cudaEventCreateWithFlags(&c->band_gev[i], cudaEventDisableTiming));
    ARC_CK(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < arc_ctx::kMaxBands; ++i) {
        ARC_CK(c, cudaStreamCreateWithFlags(&c->band_stream[i], cudaStreamNonBlocking));
        ARC_CK(c, cudaEventCreateWithFlags(&c->band_ev[i], cudaEventDisableTiming));
    }
    ARC_CK(c, cudaEventCreateWithFlags(&c->copies_done, cudaEventDisableTiming));
    ARC_CK(c, cudaEventCreateWithFlags(&c->frame_start, cudaEventDisableTiming));
    return ARC_OK;
}

// First row of band b of n (b = n: the height). The bands' heights go 4 : ... : 4 : 2 : 1, so the
// last band, the only one whose copies follow the traversal, is short (1080 rows in 8 bands: six of
// 160 rows, then 80 and 40, each a whole number of the kernels' 16- and 8-row blocks).
static uint32_t band_edge(uint32_t height, uint32_t b, uint32_t n) {
    auto weight = [n](uint32_t i) -> uint64_t { return i + 2u < n ? 4u : (i + 2u == n ? 2u : 1u); };
    uint64_t before = 0, total = 0;
    for (uint32_t i = 0; i < n; ++i) {
        if (i < b) before += weight(i);
        total += weight(i);
    }
    return (uint32_t)((uint64_t)height * before / total);
}

// Host-buffer frame in horizontal bands (band_edge): the copy stream waits for each band and copies
// that band's rows of every output while later bands trace, so only the last band's copies follow the
// traversal. The plain kernel's bands are launched together on their own streams (the SMs fill with
// band b + 1 while band b drains: no tail per band); the persistent kernel's bands share its queue
// head and run one after another on the context's stream.
int arc_trace_frame(arc_ctx* c, uint32_t width, uint32_t height, uint32_t* gdm, uint32_t* gnm, uint32_t* gaa,
                    arc_hit_record* hits, arc_hit_record* gi_hits, uint64_t* n_gi_out) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if ((rc = check_dims(c, width, height))) return rc;
    if (!gdm || !gnm || !gaa) return set_err(c, ARC_E_INVALID_ARG, "null G-buffer");
    if ((rc = ensure_band_streams(c))) return rc;
    const bool surf = c->surface_mats[0] || cam_underwater(c->cam);
    if (surf && (rc = arc_ctx_reserve_surface(c, (size_t)width * height))) return rc;
    const size_t np = (size_t)width * height;
    void* host[5] = {gdm, gnm, gaa, hits, gi_hits};
    const size_t px_bytes[5] = {8, 8, 4, 20, 20};
    size_t total = 0;
    size_t off[5];
    for (int i = 0; i < 5; ++i) {
        off[i] = total;
        if (host[i]) total += (np * px_bytes[i] + 255) & ~(size_t)255;
    }
    void* stage;
    if ((rc = arc_ctx_stage(c, total, &stage))) return rc;
    unsigned char* base = static_cast<unsigned char*>(stage);
    unsigned char* dev[5];
    for (int i = 0; i < 5; ++i) dev[i] = host[i] ? base + off[i] : nullptr;
    arc::FrameParams P = frame_params(c, width, height);
    P.gbuf_depth_mat = reinterpret_cast<uint32_t*>(dev[0]);
    P.gbuf_norm_motion = reinterpret_cast<uint32_t*>(dev[1]);
    P.gbuf_albedo_ao = reinterpret_cast<uint32_t*>(dev[2]);
    P.hits = reinterpret_cast<arc_hit_record*>(dev[3]);
    P.gi_hits = reinterpret_cast<arc_hit_record*>(dev[4]);
    P.do_gi = 1;
    const bool concurrent = c->cfg.variant == 0u;
    const uint32_t n_bands =
        std::max<uint32_t>(1u, std::min<uint32_t>((uint32_t)arc_ctx::kMaxBands, height / (concurrent ? 128u : 256u)));
    ARC_CK(c, cudaMemsetAsync(c->d_scratch, 0, sizeof(Scratch), c->stream));
    if (surf) ARC_CK(c, cudaMemsetAsync(c->d_surf_count, 0, sizeof(uint32_t) * arc_ctx::kMaxBands, c->stream));
    ARC_CK(c, cudaEventRecord(c->ev0, c->stream));
    ARC_CK(c, cudaEventRecord(c->frame_start, c->stream));
    for (uint32_t b = 0; b < n_bands; ++b) {
        const uint32_t r0 = band_edge(height, b, n_bands), r1 = band_edge(height, b + 1u, n_bands);
        frame_rows(c, P, r0, r1);
        cudaStream_t st = c->stream;
        if (concurrent) {
            st = c->band_stream[b];
            ARC_CK(c, cudaStreamWaitEvent(st, c->frame_start, 0));
        } else if (b > 0) {
            ARC_CK(c, cudaMemsetAsync(&c->d_scratch->queue_head, 0, sizeof(uint32_t), c->stream));
        }
        if ((rc = surface_prepare(c, P, c->d_surf_count + b))) return rc;
        // the surface branches run between the primary kernel and the GI pass, so the band's G-buffer and
        // primary hit records are final (band_gev) and copied while its GI pass runs
        const arc::FrameHooks hooks{true, c->band_gev[b]};
        ARC_CK(c, arc::launch_frame(P, c->cam, c->cfg, c->n_sm, st, &hooks));
        ARC_CK(c, cudaEventRecord(c->band_ev[b], st));
        ARC_CK(c, cudaStreamWaitEvent(c->copy_stream, c->band_gev[b], 0));
        ARC_CK(c, cudaStreamWaitEvent(c->gi_copy_stream, c->band_ev[b], 0));
        for (int i = 0; i < 5; ++i) {
            if (!host[i]) continue;
            const size_t o = (size_t)r0 * width * px_bytes[i], len = (size_t)(r1 - r0) * width * px_bytes[i];
            ARC_CK(c, cudaMemcpyAsync(static_cast<unsigned char*>(host[i]) + o, dev[i] + o, len, cudaMemcpyDeviceToHost,
                                      i == 4 ? c->gi_copy_stream : c->copy_stream));
        }
    }
    if (concurrent)
        for (uint32_t b = 0; b < n_bands; ++b) ARC_CK(c, cudaStreamWaitEvent(c->stream, c->band_ev[b], 0));
    ARC_CK(c, cudaEventRecord(c->ev1, c->stream));
    c->timing_pending = true;
    ARC_CK(c, cudaEventRecord(c->copies_done, c->copy_stream));
    ARC_CK(c, cudaEventRecord(c->gi_copies_done, c->gi_copy_stream));
    ARC_CK(c, cudaStreamWaitEvent(c->stream, c->copies_done, 0));
    ARC_CK(c, cudaStreamWaitEvent(c->stream, c->gi_copies_done, 0));
    return collect_frame(c, np, n_gi_out);
}

int arc_trace_primary(arc_ctx* c, uint32_t width, uint32_t height, uint32_t* gdm, uint32_t* gnm, uint32_t* gaa,
                      arc_hit_record* hits) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if ((rc = check_dims(c, width, height))) return rc;
    if (!gdm || !gnm || !gaa) return set_err(c, ARC_E_INVALID_ARG, "null G-buffer");
    const size_t np = (size_t)width * height;
    const size_t b_g = np * 20, b_h = hits ? np * 20 : 0;
    void* stage;
    if ((rc = arc_ctx_stage(c, b_g + b_h, &stage))) return rc;
    unsigned char* base = static_cast<unsigned char*>(stage);
    uint32_t* d_gdm = reinterpret_cast<uint32_t*>(base);
    uint32_t* d_gnm = reinterpret_cast<uint32_t*>(base + np * 8);
    uint32_t* d_gaa = reinterpret_cast<uint32_t*>(base + np * 16);
    arc_hit_record* d_hits = hits ? reinterpret_cast<arc_hit_record*>(base + b_g) : nullptr;
    if ((rc = arc_trace_primary_dev(c, width, height, d_gdm, d_gnm, d_gaa, d_hits))) return rc;
    ARC_CK(c, cudaMemcpyAsync(gdm, d_gdm, np * 8, cudaMemcpyDeviceToHost, c->stream));
    ARC_CK(c, cudaMemcpyAsync(gnm, d_gnm, np * 8, cudaMemcpyDeviceToHost, c->stream));
    ARC_CK(c, cudaMemcpyAsync(gaa, d_gaa, np * 4, cudaMemcpyDeviceToHost, c->stream));
    if (hits) ARC_CK(c, cudaMemcpyAsync(hits, d_hits, b_h, cudaMemcpyDeviceToHost, c->stream));
    return collect_frame(c, np, nullptr);
}

int arc_trace_secondary(arc_ctx* c, uint32_t width, uint32_t height, const uint32_t* gdm, const uint32_t* gnm,
                        arc_hit_record* gi_hits) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if ((rc = check_dims(c, width, height))) return rc;
    if (!gdm || !gnm || !gi_hits) return set_err(c, ARC_E_INVALID_ARG, "null buffer");
    const size_t np = (size_t)width * height;
    void* stage;
    if ((rc = arc_ctx_stage(c, np * 36, &stage))) return rc;
    unsigned char* base = static_cast<unsigned char*>(stage);
    uint32_t* d_gdm = reinterpret_cast<uint32_t*>(base);
    uint32_t* d_gnm = reinterpret_cast<uint32_t*>(base + np * 8);
    arc_hit_record* d_hits = reinterpret_cast<arc_hit_record*>(base + np * 16);
    ARC_CK(c, cudaMemcpyAsync(d_gdm, gdm, np * 8, cudaMemcpyHostToDevice, c->stream));
    ARC_CK(c, cudaMemcpyAsync(d_gnm, gnm, np * 8, cudaMemcpyHostToDevice, c->stream));
    if ((rc = arc_trace_secondary_dev(c, width, height, d_gdm, d_gnm, d_hits))) return rc;
    ARC_CK(c, cudaMemcpyAsync(gi_hits, d_hits, np * 20, cudaMemcpyDeviceToHost, c->stream));
    return arc_ctx_finish(c);
}

int arc_trace_rays_dev(arc_ctx* c, const arc_ray* rays, uint32_t n, float max_dist_m, uint32_t lod_bias, int ignore_water,
                       arc_hit_record* hits) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (n && (!rays || !hits)) return set_err(c, ARC_E_INVALID_ARG, "null buffer");
    if (lod_bias > 2u) return set_err(c, ARC_E_INVALID_ARG, "lod_bias must be 0, 1 or 2");
    ARC_CK(c, arc::launch_rays(c->world(), c->cam, rays, n, max_dist_m, lod_bias, ignore_water, hits, c->stream));
    return ARC_OK;
}

int arc_trace_rays(arc_ctx* c, const arc_ray* rays, uint32_t n, float max_dist_m, uint32_t lod_bias, int ignore_water,
                   arc_hit_record* hits) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (n == 0) return ARC_OK;
    if (!rays || !hits) return set_err(c, ARC_E_INVALID_ARG, "null buffer");
    void* stage;
    if ((rc = arc_ctx_stage(c, (size_t)n * 44, &stage))) return rc;
    arc_ray* d_rays = static_cast<arc_ray*>(stage);
    arc_hit_record* d_hits = reinterpret_cast<arc_hit_record*>(static_cast<unsigned char*>(stage) + (size_t)n * 24);
    ARC_CK(c, cudaMemcpyAsync(d_rays, rays, (size_t)n * 24, cudaMemcpyHostToDevice, c->stream));
    if ((rc = arc_trace_rays_dev(c, d_rays, n, max_dist_m, lod_bias, ignore_water, d_hits))) return rc;
    ARC_CK(c, cudaMemcpyAsync(hits, d_hits, (size_t)n * 20, cudaMemcpyDeviceToHost, c->stream));
    return arc_ctx_finish(c);
}

// ------------------------------------------------------------------------------------------------
// Batched views: many cameras over several worlds in one persistent launch, optionally replayed
// from a captured CUDA graph (memset of the scratch, upload of the view table from a pinned mirror,
// the kernel, and the GI-count copy). A new graph is captured when the view count, the GI-count
// destination or the launch configuration changes; otherwise the frame only rewrites the mirror.
// ------------------------------------------------------------------------------------------------

static int views_prepare(arc_ctx* c, const arc_view_desc* views, uint32_t n, uint32_t* queue_len) {
    if (!c || !views || n == 0) return set_err(c, ARC_E_INVALID_ARG, "no views");
    if (!c->have_world) return set_err(c, ARC_E_NO_WORLD, "no world uploaded");
    if (n > c->views_cap) {
        cudaFree(c->d_views);
        if (c->h_views) cudaFreeHost(c->h_views);
        c->d_views = nullptr;
        c->h_views = nullptr;
        c->views_cap = 0;
        ARC_CK(c, cudaMalloc((void**)&c->d_views, sizeof(arc::ViewDev) * n));
        ARC_CK(c, cudaMallocHost((void**)&c->h_views, sizeof(arc::ViewDev) * n));
        c->views_cap = n;
        if (c->views_exec) cudaGraphExecDestroy(c->views_exec);
        if (c->views_graph) cudaGraphDestroy(c->views_graph);
        c->views_exec = nullptr;
        c->views_graph = nullptr;
    }
    ARC_CK(c, cudaStreamSynchronize(c->stream));  // the previous launch has read the mirror
    // surface list over every view's pixels when a view's world holds water or mirror voxels or a
    // view's camera is under water
    bool surf = false;
    uint64_t n_px = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t slot = views[i].world_slot;
        if (slot < (uint32_t)arc_ctx::kSlots && (c->surface_mats[slot] || cam_underwater(views[i].cam))) surf = true;
        n_px += (uint64_t)views[i].width * views[i].height;
    }
    if (surf && n_px > 0xFFFFFFFFull) return set_err(c, ARC_E_CAPACITY, "batch above 2^32 pixels");
    if (surf) {
        int rc = arc_ctx_reserve_surface(c, (size_t)n_px);
        if (rc) return rc;
    }
    c->views_surf_cap = surf ? (uint32_t)n_px : 0u;
    uint64_t q = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const arc_view_desc& d = views[i];
        const uint32_t slot = d.world_slot;
        if (slot >= (uint32_t)arc_ctx::kSlots) return set_err(c, ARC_E_INVALID_ARG, "view world slot out of range");
        const uint32_t* g = slot == 0 ? c->grid : c->slots[slot].grid;
        if (slot != 0 && !c->slots[slot].valid) return set_err(c, ARC_E_NO_WORLD, "view names an empty world slot");
        if (d.cam.world_grid_dims[0] != g[0] || d.cam.world_grid_dims[1] != g[1] || d.cam.world_grid_dims[2] != g[2])
            return set_err(c, ARC_E_INVALID_ARG, "view camera grid differs from its world");
        if (d.width == 0 || d.height == 0 || (d.cam.world_grid_dims[3] & 0xFFFFu) != d.width ||
            (d.cam.world_grid_dims[3] >> 16) != d.height)
            return set_err(c, ARC_E_INVALID_ARG, "view size differs from its camera world_grid_dims.w");
        if (!d.gbuf_depth_mat || !d.gbuf_norm_motion || !d.gbuf_albedo_ao) return set_err(c, ARC_E_INVALID_ARG, "null G-buffer");
        if (slot == 0 && c->n_bodies && ((d.cam.point_light_count[1] >> 16) & 0xFFFFu))
            return set_err(c, ARC_E_INVALID_ARG, "batched views do not trace rigid bodies (use arc_trace_frame_dev)");
        arc::ViewDev& v = c->h_views[i];
        memset(&v, 0, sizeof v);
        v.cam = d.cam;
        v.slot = slot;
        v.width = d.width;
        v.height = d.height;
        v.tiles_x = (d.width + c->cfg.tile_w - 1u) / c->cfg.tile_w;
        v.queue_begin = (uint32_t)q;
        v.gbuf_depth_mat = d.gbuf_depth_mat;
        v.gbuf_norm_motion = d.gbuf_norm_motion;
        v.gbuf_albedo_ao = d.gbuf_albedo_ao;
        v.hits = d.hits;
        v.gi_hits = d.gi_hits;
        v.view_id = i;
        if (surf) {
            v.surf = c->d_surf;
            v.surf_count = &c->d_scratch->surf_count;
            v.surf_cap = (uint32_t)n_px;
        }
        uint64_t tx = v.tiles_x, ty = (d.height + c->cfg.tile_h - 1u) / c->cfg.tile_h;
        if (c->cfg.order == 1u) {  // whole super-tiles of 8 x 8 tiles; the padding tiles map off the view
            tx = (tx + 7u) & ~7ull;
            ty = (ty + 7u) & ~7ull;
        }
        q += tx * ty * 32u;
        if (q > (1ull << 31)) return set_err(c, ARC_E_CAPACITY, "batch exceeds 2^31 queue entries");
    }
    *queue_len = (uint32_t)q;
    return ARC_OK;
}

static int views_enqueue(arc_ctx* c, uint32_t n, uint32_t queue_len, uint64_t* n_gi_dev) {
    arc::ViewsParams V;
    V.views = c->d_views;
    V.n_views = n;
    V.worlds = c->d_worlds;
    V.scratch = c->d_scratch;
    V.queue_len = queue_len;
    V.tile_w = c->cfg.tile_w;
    V.tile_h = c->cfg.tile_h;
    V.refill_threshold = c->cfg.refill_threshold;
    V.surf = c->views_surf_cap ? 1u : 0u;
    V.gi_split = c->cfg.variant == 0u ? 1u : 0u;
    V.order = c->cfg.order;
    ARC_CK(c, cudaMemsetAsync(c->d_scratch, 0, sizeof(arc::Scratch), c->stream));
    ARC_CK(c, cudaMemcpyAsync(c->d_views, c->h_views, sizeof(arc::ViewDev) * n, cudaMemcpyHostToDevice, c->stream));
    ARC_CK(c, arc::launch_views(V, c->cfg, c->n_sm, c->stream));
    if (c->views_surf_cap)
        ARC_CK(c, arc::launch_surface_views(V, c->d_surf, &c->d_scratch->surf_count, c->views_surf_cap, c->n_sm, c->stream));
    if (n_gi_dev)
        ARC_CK(c, cudaMemcpyAsync(n_gi_dev, &c->d_scratch->gi_rays, sizeof(uint64_t), cudaMemcpyDeviceToDevice, c->stream));
    return ARC_OK;
}

int arc_trace_views_dev(arc_ctx* c, const arc_view_desc* views, uint32_t n_views, uint64_t* n_gi_dev, int use_graph) {
    uint32_t queue_len = 0;
    int rc = views_prepare(c, views, n_views, &queue_len);
    if (rc) return rc;
    ARC_CK(c, cudaEventRecord(c->ev0, c->stream));
    if (!use_graph) {
        if ((rc = views_enqueue(c, n_views, queue_len, n_gi_dev))) return rc;
    } else {
        const bool same = c->views_exec && c->graph_n_views == n_views && c->graph_n_gi == n_gi_dev &&
                          c->graph_queue_len == queue_len && c->graph_surf_cap == c->views_surf_cap &&
                          c->graph_surf_list == c->d_surf && memcmp(&c->graph_cfg, &c->cfg, sizeof c->cfg) == 0;
        if (!same) {
            if (c->views_exec) cudaGraphExecDestroy(c->views_exec);
            if (c->views_graph) cudaGraphDestroy(c->views_graph);
            c->views_exec = nullptr;
            c->views_graph = nullptr;
            ARC_CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            rc = views_enqueue(c, n_views, queue_len, n_gi_dev);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
            c->views_graph = g;
            ARC_CK(c, cudaGraphInstantiate(&c->views_exec, g, 0));
            c->graph_n_views = n_views;
            c->graph_n_gi = n_gi_dev;
            c->graph_queue_len = queue_len;
            c->graph_surf_cap = c->views_surf_cap;
            c->graph_surf_list = c->d_surf;
            c->graph_cfg = c->cfg;
        }
        ARC_CK(c, cudaGraphLaunch(c->views_exec, c->stream));
    }
    ARC_CK(c, cudaEventRecord(c->ev1, c->stream));
    c->timing_pending = true;
    return ARC_OK;
}

int arc_autotune_views_dev(arc_ctx* c, const arc_view_desc* views, uint32_t n_views, uint32_t frames,
                           arc_launch_config* best_out, float* best_ms) {
    if (!c) return ARC_E_INVALID_ARG;
    if (frames == 0) frames = 3;
    // the plain kernel + GI pass over register budget x block size x tile shape x tile order; the
    // persistent kernel (variant 1) lost every measured batch by 1.6x or more and stays out of the
    // space (arc_set_launch_config still selects it)
    std::vector<arc_launch_config> cands;
    for (uint32_t rb : {2u, 3u, 4u})
        for (uint32_t bt : {128u, 256u})
            for (uint32_t tw : {8u, 4u, 16u})
                for (uint32_t order : {0u, 1u}) cands.push_back(arc_launch_config{0u, bt, 0u, tw, 32u / tw, 8u, rb, order, 0u});
    const arc_launch_config saved = c->cfg;
    float best = 1e30f;
    arc_launch_config best_cfg = saved;
    std::vector<float> ms(frames);
    int rc = ARC_OK;
    for (const arc_launch_config& cfg : cands) {
        c->cfg = cfg;
        for (uint32_t f = 0; f <= frames && !rc; ++f) {
            rc = arc_trace_views_dev(c, views, n_views, nullptr, 0);
            if (rc) break;
            cudaEventSynchronize(c->ev1);
            float t = 0.0f;
            cudaEventElapsedTime(&t, c->ev0, c->ev1);
            if (f) ms[f - 1] = t;
        }
        if (rc) break;
        std::sort(ms.begin(), ms.end());
        if (ms[frames / 2] < best) {
            best = ms[frames / 2];
            best_cfg = cfg;
        }
    }
    c->cfg = rc ? saved : best_cfg;
    if (rc) return rc;
    if (best_out) *best_out = best_cfg;
    if (best_ms) *best_ms = best;
    return arc_ctx_finish(c);
}

// Autotuner: times each candidate launch configuration on the caller's frame (median of `frames`
// launches after one warm-up, CUDA events on the context stream) and installs the fastest.
int arc_autotune_frame_dev(arc_ctx* c, uint32_t width, uint32_t height, uint32_t* gdm, uint32_t* gnm, uint32_t* gaa,
                           arc_hit_record* hits, arc_hit_record* gi_hits, uint32_t frames, arc_launch_config* best_out,
                           float* best_ms) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if ((rc = check_dims(c, width, height))) return rc;
    if (!gdm || !gnm || !gaa) return set_err(c, ARC_E_INVALID_ARG, "null G-buffer");
    if (frames == 0) frames = 3;
    // candidates: the plain kernel + GI pass over register budget x block size x block order (row-major
    // or Morton super-tiles) x traversal loop (descent loop or one node per iteration, budgets 2 and 3),
    // and the persistent queue kernel at its best-measured settings
    std::vector<arc_launch_config> cands;
    for (uint32_t rb : {3u, 4u})
        for (uint32_t thr : {16u, 24u}) cands.push_back(arc_launch_config{1u, 256u, 0u, 8u, 4u, thr, rb, 0u, 0u});
    for (uint32_t rb : {2u, 3u, 4u})
        for (uint32_t bt : {64u, 128u, 256u})
            for (uint32_t order : {0u, 1u})
                for (uint32_t feat : {0u, ARC_FEAT_NODE_VISIT, ARC_FEAT_GI_SORT}) {
                    if (feat == ARC_FEAT_NODE_VISIT && rb == 4u) continue;
                    cands.push_back(arc_launch_config{0u, bt, 0u, 8u, 4u, 8u, rb, order, feat});
                }
    const arc_launch_config saved = c->cfg;
    float best = 1e30f;
    arc_launch_config best_cfg = saved;
    std::vector<float> ms(frames);
    for (const arc_launch_config& cfg : cands) {
        c->cfg = cfg;
        for (uint32_t f = 0; f <= frames; ++f) {
            if ((rc = arc_trace_frame_dev(c, width, height, gdm, gnm, gaa, hits, gi_hits, nullptr))) {
                c->cfg = saved;
                return rc;
            }
            ARC_CK(c, cudaEventSynchronize(c->ev1));
            float t = 0.0f;
            ARC_CK(c, cudaEventElapsedTime(&t, c->ev0, c->ev1));
            if (f) ms[f - 1] = t;
        }
        std::sort(ms.begin(), ms.end());
        const float med = ms[frames / 2];
        if (med < best) {
            best = med;
            best_cfg = cfg;
        }
    }
    c->cfg = best_cfg;
    if (best_out) *best_out = best_cfg;
    if (best_ms) *best_ms = best;
    return arc_ctx_finish(c);
}

int arc_shadow_rays_di_dev(arc_ctx* c, const arc_ray* rays, const float* max_dist_m, uint32_t n, float* vis) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (n && (!rays || !max_dist_m || !vis)) return set_err(c, ARC_E_INVALID_ARG, "null buffer");
    if (n) ARC_CK(c, arc::launch_shadow_di(c->world(), c->cam, rays, max_dist_m, n, vis, c->stream));
    return ARC_OK;
}

int arc_set_rigid_bodies(arc_ctx* c, const arc_rigid_body* bodies, uint32_t n) {
    int rc = arc_ctx_check_ready(c, false);
    if (rc) return rc;
    if (n > ARC_MAX_RIGID_BODIES) return set_err(c, ARC_E_INVALID_ARG, "more than 32 rigid bodies");
    if (n && !bodies) return set_err(c, ARC_E_INVALID_ARG, "null body table");
    for (uint32_t i = 0; i < n; ++i) {
        const arc_rigid_body& b = bodies[i];
        uint32_t root;
        memcpy(&root, &b.local_bounds_and_root[3], 4);
        bool ok = root == ARC_EMPTY_CHUNK || root < c->n_nodes;
        for (int k = 0; k < 3; ++k)
            ok = ok && std::isfinite(b.local_bounds_and_root[k]) && b.local_bounds_and_root[k] > 0.0f &&
                 b.local_bounds_and_root[k] <= 16.0f;
        for (int k = 0; k < 16; ++k)
            ok = ok && std::isfinite(b.world_to_local[k]) && std::isfinite(b.local_to_world[k]) &&
                 std::isfinite(b.prev_local_to_world[k]);
        for (int k = 0; k < 4; ++k) ok = ok && std::isfinite(b.world_sphere[k]);
        if (!ok) {
            char m[160];
            snprintf(m, sizeof m, "rigid body %u: root out of the node pool, local bounds outside (0, 16] m or a non-finite value", i);
            return set_err(c, ARC_E_INVALID_ARG, m);
        }
    }
    if (!c->d_bodies) ARC_CK(c, cudaMalloc((void**)&c->d_bodies, sizeof(arc_rigid_body) * ARC_MAX_RIGID_BODIES));
    ARC_CK(c, cudaStreamSynchronize(c->stream));
    if (n) ARC_CK(c, cudaMemcpy(c->d_bodies, bodies, sizeof(arc_rigid_body) * n, cudaMemcpyHostToDevice));
    c->n_bodies = n;
    return arc_ctx_sync_world_table(c);
}

int arc_trace_rigid_bodies_dev(arc_ctx* c, const arc_ray* rays, uint32_t n, float max_dist_m, arc_hit_record* hits,
                               float* detail) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (n && (!rays || !hits)) return set_err(c, ARC_E_INVALID_ARG, "null buffer");
    if (n) ARC_CK(c, arc::launch_rigid_rays(c->world(), c->cam, rays, n, max_dist_m, hits, detail, c->stream));
    return ARC_OK;
}

int arc_shadow_rays_dev(arc_ctx* c, const arc_ray* rays, uint32_t n, float max_dist_m, float* vis) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (n && (!rays || !vis)) return set_err(c, ARC_E_INVALID_ARG, "null buffer");
    ARC_CK(c, arc::launch_shadow(c->world(), c->cam, rays, n, max_dist_m, vis, c->stream));
    return ARC_OK;
}

}  // extern "C"
