// Library-internal host interface between the world stages (hc_gb300.cu) and the request server
// (hc_server.cpp). Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/hc_gb300.h"

namespace hc {
namespace detail {

// Indices into the world's device counter words.
enum : int { kWorldCountDirty = 0, kWorldCountRemesh = 4, kWorldCountWords = 8 };

// Each enqueues work on `st` and reads nothing back.
hc_status world_enqueue_edits(hc_world *w, const hc_edit *d_edits, uint32_t n, cudaStream_t st);
hc_status world_enqueue_heights(hc_world *w, cudaStream_t st);
// positions: device int32 x 3n; slots: device int32 x n
hc_status world_enqueue_place(hc_world *w, const int32_t *d_pos, const int32_t *d_slots, uint32_t n, cudaStream_t st);
hc_status world_enqueue_evict(hc_world *w, const int32_t *d_pos, uint32_t n, cudaStream_t st);
// Stored edits of n loaded chunks (slots, offsets and entries on the device), applied in order.
hc_status world_enqueue_deltas(hc_world *w, const int32_t *d_slots, const uint32_t *d_boff, const uint32_t *d_soff,
                               const uint32_t *d_blocks, const uint16_t *d_suns, uint32_t n, cudaStream_t st);
// The remesh list lands in world_remesh_list (length counts[kWorldCountRemesh]).
hc_status world_enqueue_remesh(hc_world *w, const hc_batch_arena *arena, cudaStream_t st);
// Draw records of the last remesh's meshes (d_pos: 3 int32 per grid cell of scratch).
hc_status world_enqueue_infos(hc_world *w, const hc_batch_arena *arena, int32_t *d_pos, hc_mesh_info *d_infos,
                              cudaStream_t st);

const uint32_t *world_counts(const hc_world *w);           // device
const int32_t *world_remesh_list(const hc_world *w);       // device
const unsigned long long *world_state(const hc_world *w); // device: quad cursor, mesh cursor, work, failed
hc_pool *world_pool(const hc_world *w);
size_t pool_planes_bytes_per_slot();

hc_status ctx_fail(hc_ctx *ctx, hc_status s, const std::string &msg);
int ctx_device(const hc_ctx *ctx);

} // namespace detail
} // namespace hc
