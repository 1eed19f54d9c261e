// arc_ctx.h — the opaque arc_ctx behind the C ABI (one device, one stream).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "arc_kernels.h"

struct arc_ctx {
    int device = 0;
    int n_sm = 0;
    cudaStream_t stream = nullptr;

    // Group-0 pools (device copies of WorldMap's packed buffers)
    uint32_t grid[3] = {0, 0, 0};
    uint32_t n_roots = 0;
    uint32_t* d_roots = nullptr;
    arc_node64* d_nodes = nullptr;
    uint32_t n_nodes = 0, cap_nodes = 0;
    arc_brick64* d_bricks = nullptr;
    uint32_t n_bricks = 0, cap_bricks = 0;
    arc_material* d_palette = nullptr;
    bool have_world = false;

    arc_camera_uniforms cam{};
    bool have_cam = false;

    // rigid voxel bodies (GpuRigidBodyInstance table; their trees live in the node pool above)
    arc_rigid_body* d_bodies = nullptr;
    uint32_t n_bodies = 0;

    // extra worlds for batched multi-view launches (slot 0 is the world above)
    static constexpr int kSlots = 8;
    struct Slot {
        uint32_t grid[3] = {0, 0, 0};
        uint32_t n_roots = 0, n_nodes = 0, n_bricks = 0;
        uint32_t* d_roots = nullptr;
        arc_node64* d_nodes = nullptr;
        arc_brick64* d_bricks = nullptr;
        arc_material* d_palette = nullptr;
        bool valid = false;
    } slots[kSlots];
    arc::World* d_worlds = nullptr;  // device table of kSlots World records

    // batched views: device table, pinned host mirror, captured graph
    arc::ViewDev* d_views = nullptr;
    arc::ViewDev* h_views = nullptr;
    uint32_t views_cap = 0;
    cudaGraph_t views_graph = nullptr;
    cudaGraphExec_t views_exec = nullptr;
    uint32_t graph_n_views = 0, graph_queue_len = 0;
    uint64_t* graph_n_gi = nullptr;
    arc_launch_config graph_cfg{};

    arc::Scratch* d_scratch = nullptr;
    uint32_t* d_status = nullptr;
    uint32_t last_status = 0;

    // staging block of the host-buffer entry points
    void* d_stage = nullptr;
    size_t stage_bytes = 0;
    // scratch of the globally sorted GI pass (ARC_FEAT_GI_SORT): bins, per-pixel rays, sorted rays
    unsigned char* d_gisort = nullptr;
    size_t gisort_bytes = 0;
    // table of the top two tree levels (ARC_FEAT_TOP_TABLE), rebuilt on the device before every frame
    unsigned char* d_top = nullptr;

    // SHARC cache
    uint32_t* d_sharc_keys = nullptr;
    uint32_t* d_sharc_accum = nullptr;
    arc_sharc_slot* d_sharc_resolved = nullptr;
    void* d_sharc_stage = nullptr;
    size_t sharc_stage_bytes = 0;
    uint32_t sharc_mode = 0;  // 0 reference shading, 1 one-bounce estimator of the cache comparison

    // neural radiance cache: FP32 masters, Adam moments, gradient (contiguous), FP16 layouts, loss
    float* d_nrc_w32 = nullptr;
    float* d_nrc_m = nullptr;
    float* d_nrc_v = nullptr;
    float* d_nrc_grad = nullptr;
    void* d_nrc_w16 = nullptr;
    float* d_nrc_ema = nullptr;       // exponential moving average of the weights (inference)
    void* d_nrc_w16_ema = nullptr;    // its FP16 forward layout (mma.sync kernels)
    void* d_nrc_wu_ema = nullptr;     // its FP16 tensor-core operand layout (tcgen05 kernels)
    void* d_nrc_wu = nullptr;         // the latest weights in the tensor-core layout (tcgen05 training)
    int nrc_infer_path = 3;           // tcgen05 inference: 1 one tile group, 2 four, 3 automatic; 0 = mma.sync
    int nrc_train_path = 1;           // 1 = tcgen05 training, 0 = mma.sync training
    float nrc_ema_decay = 0.99f;
    uint32_t nrc_ema_warmup = 0;      // EMA warm-up: decay min(nrc_ema_decay, (1 + k) / (warmup + k)); 0 = off
    bool nrc_clamp = false;           // queries return max(output, 0)
    float nrc_beta1 = 0.9f, nrc_beta2 = 0.99f;  // Adam moment decays
    bool cache_pdl = true;            // radiance-cache kernels launched with programmatic dependent launch
    uint32_t nrc_sample_cluster = 1;  // training samples in runs of this many consecutive hit-list entries
    float* d_nrc_loss = nullptr;
    uint32_t nrc_step = 0;
    // in-place edits: device counters [next node, next brick, bricks rewritten, overflow] and staging
    uint32_t* d_edit = nullptr;
    void* d_edit_stage = nullptr;
    void* h_edit_stage = nullptr;
    size_t edit_stage_bytes = 0;

    // per-frame training batch of arc_nrc_train_frame_dev: inputs (9 floats) + targets (3), and the
    // gate word (the batch size, 0 when the frame has no GI hit) that the training kernels read
    float* d_nrc_batch = nullptr;
    uint32_t nrc_batch_cap = 0;
    uint32_t* d_nrc_gate = nullptr;

    // primary-pass surface list: hits that take the underwater / water / mirror branch, listed by the
    // frame kernels and shaded by the surface kernel (entries for every pixel of the largest frame or
    // batch so far; kMaxBands counters for the bands of a host-buffer frame). surface_mats[s] is set
    // when world slot s may hold water or mirror voxels (upload, patch or edit); a frame without them
    // and with the camera above water skips the list.
    arc::SurfaceEntry* d_surf = nullptr;
    uint32_t* d_surf_count = nullptr;
    size_t surf_cap = 0;
    bool surface_mats[kSlots] = {};
    uint32_t views_surf_cap = 0;                   // list entries of the current view batch (0: no list)
    uint32_t graph_surf_cap = 0;                   // ... and of the captured batch graph
    arc::SurfaceEntry* graph_surf_list = nullptr;  // the list the captured graph writes

    // fault-injection hooks (arc_debug_set): the cycle budget of each tensor-core mbarrier wait
    // (0 = the default of about one second), NRC kernels whose weight barrier is armed but never fed
    // (so the wait runs out), and an upload that skips the pool range validation
    long long tc_wait_budget = 0;
    bool tc_stall = false;
    bool skip_pool_validation = false;

    arc_launch_config cfg{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // host-buffer frames: copy stream and per-band events (copies of a band overlap the next band)
    static constexpr int kMaxBands = 8;
    static constexpr uint32_t kDefaultFrameBands = 4;  // device frames (arc_set_frame_bands 0)
    uint32_t frame_bands = 0;                           // arc_set_frame_bands; 0 = kDefaultFrameBands
    cudaStream_t copy_stream = nullptr;        // G-buffer and primary hit record copies, band by band
    cudaStream_t gi_copy_stream = nullptr;     // GI hit record copies, band by band
    cudaStream_t band_stream[kMaxBands] = {};  // the plain kernel's bands run concurrently, one per stream
    cudaEvent_t band_ev[kMaxBands] = {};       // a band's kernels done
    cudaEvent_t band_gev[kMaxBands] = {};      // a band's G-buffer and primary hit records final
    cudaEvent_t copies_done = nullptr, gi_copies_done = nullptr, frame_start = nullptr;
    // side stream for a cache query that overlaps the cache's own update (arc_nrc_frame_dev,
    // arc_sharc_frame_dev): forked from and joined back into `stream` with two events
    cudaStream_t side_stream = nullptr;
    cudaEvent_t side_fork = nullptr, side_join = nullptr;
    bool timing_pending = false;
    float last_ms = 0.0f;
    uint64_t last_rays = 0;
    std::string err;

    arc::World world() const;
};

// Launch on the context's stream with programmatic stream serialization when c->cache_pdl is set: the
// kernel is scheduled while the kernel ahead of it finishes and waits for it (griddepcontrol.wait,
// a hardware wait) before it reads that kernel's results.
template <typename... KArgs, typename... Args>
cudaError_t arc_launch_overlapped(const arc_ctx* c, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                  Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = c->cache_pdl ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, static_cast<Args&&>(args)...);
}

int arc_ctx_check_ready(arc_ctx* c, bool need_cam);
int arc_ctx_finish(arc_ctx* c);
// edit allocator (arc_edit.cu): restart growth at the end of the uploaded pools / keep it above a patch
int arc_edit_reset(arc_ctx* c);
int arc_edit_raise_floor(arc_ctx* c, uint32_t node_floor, uint32_t brick_floor);
// NRC training samples drawn from a compacted list of GI hit points (defined with the estimator in
// arc_sharc.cu): stratified over list[0 .. *n_valid) with a seeded phase, demodulated 1-spp targets,
// interleaved into `steps` slices (n_samples a multiple of steps); gate receives n_samples, or 0
// when *n_valid is 0.
extern "C" int arc_launch_train_samples_list(arc_ctx* c, const uint32_t* list, const unsigned long long* n_valid,
                                             const float* pos, const float* nrm, const float* nrc_in, uint32_t seed,
                                             uint32_t n_samples, uint32_t steps, float* train_in, float* train_t,
                                             uint32_t* gate);
int arc_ctx_stage(arc_ctx* c, size_t bytes, void** out);
// Work enqueued between arc_ctx_side_begin and arc_ctx_side_end goes to the side stream, which first
// waits for everything enqueued on the context's stream so far; arc_ctx_side_join makes the context's
// stream wait for that side work. Between begin and end, c->stream is the side stream.
int arc_ctx_side_begin(arc_ctx* c);
int arc_ctx_side_end(arc_ctx* c);
int arc_ctx_side_join(arc_ctx* c);
// surface list of at least `entries` entries (frees and reallocates when smaller)
int arc_ctx_reserve_surface(arc_ctx* c, size_t entries);
// whether any word of the pools holds material 18 (water) or 28 (mirror) in a brick or a node payload
bool arc_pools_have_surface_mats(const arc_node64* nodes, uint32_t n_nodes, const arc_brick64* bricks, uint32_t n_bricks);
int arc_ctx_sync_world_table(arc_ctx* c);
