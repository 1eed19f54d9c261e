/*
 * arc/arc_world.h — native builder of the synthetic benchmark worlds (part of libarc_trace.so).
 *
 * Produces the three GPU pools exactly as Arcadia packs them:
 *   ChunkTree64::from_generator + build_recursive + pack_build_tree
 *     (crates/arcadia-core/src/chunk_tree/builder.rs:86-378): homogeneous-subtree collapse into
 *     uniform nodes, lod_payload averaging, BFS level-order node layout;
 *   WorldMap::rebuild_all_gpu_pools (crates/arcadia-world/src/world_map.rs:158-205): reserved empty
 *     node/brick 0, chunks appended in 3D Morton order, pointers relocated, 0xFFFFFFFF for empty chunks.
 * The scene itself (seeded value-noise heightfield + 3D value-noise caves, ids 1-16) replaces the
 * reference's generator and is this library's own definition.
 */
#ifndef ARC_WORLD_H
#define ARC_WORLD_H

#include <stdint.h>
#include "layout.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct arc_scene_desc {
    uint32_t grid[3];     /* chunks per axis */
    uint32_t seed;
    uint32_t caves;       /* 1 = carve caves */
    float cave_threshold; /* voxel empty where cave noise > threshold */
    float height_lo;      /* terrain height range, fraction of world height */
    float height_hi;
    uint32_t cave_depth;  /* caves only within this many voxels below the surface (0 = at any depth) */
} arc_scene_desc;

typedef struct arc_world_pools arc_world_pools;

/* Default 256-entry palette (crates/arcadia-core/src/material.rs:99-204). */
int arc_default_palette(arc_material* out256);
/* Builds the pools with `threads` host threads (0 = all). */
int arc_world_build(const arc_scene_desc* desc, const arc_material* palette, int threads, arc_world_pools** out);
int arc_world_info(const arc_world_pools* w, uint32_t* n_roots, uint32_t* n_nodes, uint32_t* n_bricks,
                   uint64_t* solid_voxels);
int arc_world_copy(const arc_world_pools* w, uint32_t* roots, arc_node64* nodes, arc_brick64* bricks);
int arc_world_free(arc_world_pools* w);

#ifdef __cplusplus
}
#endif

#endif /* ARC_WORLD_H */
