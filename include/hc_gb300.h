/* GB300 chunk relighter + mesher for HyperCraft: the C ABI.
 *
 * This library replaces the body of the client's per-chunk mesh task,
 *   ChunkTaskRunner<ChunkTaskType::kMesh>::Run   (client/src/ChunkMeshTask.cpp:41-127),
 * i.e. the 62^3 light-window seed (lines 49-87), the sun and torch flood fills
 * BlockLightAlgo::PropagateLight (lines 89-111, client/include/client/BlockLightAlgo.hpp:44-73) and
 * BlockMeshAlgo::Generate (lines 113-122, client/include/client/BlockMeshAlgo.hpp:494-521).
 * Its output is the std::vector<BlockMesh> that WorldRenderer::PushChunkMesh consumes
 * (client/include/client/WorldRenderer.hpp:69-87), byte for byte: the same packed 8-byte vertices
 * (client/include/client/BlockVertex.hpp:8-18), uint16 indices, per-mesh uint32 AABBs, transparent
 * flags, mesh split at 65,532 vertices and mesh order.
 *
 * Inputs follow the reference's chunk layout (client/include/client/Chunk.hpp:95-96): a chunk is
 * 32^3 uint16 blocks (raw = id | meta << 8, index x + (y*32 + z)*32) and 32^2 int8 sunlight heights
 * (index x + z*32). A call takes the 27 chunks of a neighbourhood in the reference's neighbour order
 * (common/include/common/Position.hpp:138-152; the centre chunk is index 26).
 *
 * All entry points return an hc_status. Pointers are plain host or device pointers; no type from
 * any framework appears here. A context is bound to one CUDA device; calls on one context from
 * several threads must use distinct streams.
 */
#ifndef HC_GB300_H
#define HC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hc_status {
	HC_OK = 0,
	HC_ERR_INVALID_ARG = 1,    /* null pointer, bad size or bad slot */
	HC_ERR_OUT_OF_MEMORY = 2,  /* device or pinned allocation failed */
	HC_ERR_CAPACITY = 3,       /* an output buffer is too small; the required sizes are written back */
	HC_ERR_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up */
	HC_ERR_CUDA = 5,           /* a CUDA runtime call failed; see hc_last_error */
	HC_ERR_NO_DEVICE = 6       /* no usable sm_103 device, or the kernels are not loadable */
} hc_status;

typedef struct hc_ctx hc_ctx;
typedef struct hc_pool hc_pool;

/* One mesh of the output, in reference order. Offsets count elements (vertices of 8 bytes, uint16
 * indices) from the start of the vertex / index buffer the call wrote. Index values are local to
 * the mesh, as in the reference. 48 bytes. */
typedef struct hc_mesh_desc {
	uint32_t vertex_offset;
	uint32_t vertex_count;
	uint32_t index_offset;
	uint32_t index_count;
	uint32_t aabb_min[3]; /* 1/16-voxel units, UINT32_MAX when empty (dep/AABB.hpp:11) */
	uint32_t aabb_max[3];
	uint32_t transparent; /* 1 for the transparent-pass stream */
	uint32_t chunk;       /* batch position of the chunk (0 for single-chunk calls) */
} hc_mesh_desc;

/* Output of a single-chunk call. The caller sets the three capacities and the three pointers
 * (host pointers for hc_mesh_chunk, device pointers for hc_mesh_chunk_device); the call writes
 * the counts. On HC_ERR_CAPACITY the counts hold the required sizes and nothing else is valid.
 * Vertices are two uint32 words each (x10_y10_z10_axis2, tex10_trans3_face3_ao2_sl6_tl6). */
typedef struct hc_chunk_mesh {
	uint32_t mesh_capacity, vertex_capacity, index_capacity;
	uint32_t mesh_count, vertex_count, index_count;
	hc_mesh_desc *meshes;
	uint32_t *vertices;
	uint16_t *indices;
} hc_chunk_mesh;

/* Worst case of one chunk: 720,896 quads (custom + regular faces), 45 meshes per stream. */
#define HC_CHUNK_MAX_QUADS 720896u
#define HC_CHUNK_MAX_MESHES 96u

const char *hc_status_string(hc_status s);
/* Text of the last error on this context (empty if none). */
const char *hc_last_error(const hc_ctx *ctx);

/* Creates a context on CUDA device `device`: uploads the block tables and allocates the
 * single-chunk staging and output buffers. */
hc_status hc_ctx_create(int device, hc_ctx **out);
void hc_ctx_destroy(hc_ctx *ctx);

/* Drop-in for ChunkMeshTask.cpp:48-122 with host buffers: copies the 27 chunks to the device,
 * relights the centre chunk's window, meshes it and copies the meshes back into `out` (host
 * pointers). `stream` is a cudaStream_t (NULL = the context's own stream). Synchronous. */
hc_status hc_mesh_chunk(hc_ctx *ctx, const uint16_t *const blocks[27], const int8_t *const heights[27],
                        hc_chunk_mesh *out, void *stream);

/* Same computation with every pointer on the device (blocks[i], heights[i] and out's three
 * buffers). Enqueues on `stream` and waits only to read the counts back. */
hc_status hc_mesh_chunk_device(hc_ctx *ctx, const uint16_t *const blocks[27], const int8_t *const heights[27],
                               hc_chunk_mesh *out, void *stream);

/* Relight only: the 34^3 light region the mesher reads ([-1, 32]^3 of the centre chunk; index
 * (x+1) + ((z+1) + (y+1)*34)*34; sun in the low nibble, torch in the high nibble), as produced by
 * the window flood fill of ChunkMeshTask.cpp:48-111. Device pointers throughout. */
hc_status hc_relight_chunk_device(hc_ctx *ctx, const uint16_t *const blocks[27], const int8_t *const heights[27],
                                  uint8_t *light34, void *stream);


/* ----------------------------------------------------------------------------------------------
 * Device chunk pool and batched meshing.
 *
 * The reference meshes one chunk per worker-thread task (ChunkTaskPool::Run,
 * client/src/ChunkTaskPool.cpp:87-130). Here chunks stay resident in a device pool of slots and
 * a batch names, per chunk to mesh, its 27 neighbour slots (neighbour order, centre last). The
 * batched form runs one persistent kernel whose CTAs take chunks from a device work counter;
 * the plain form launches the single-chunk kernel once per chunk. Both write each chunk's meshes
 * to the same arena layout, byte-identical to hc_mesh_chunk.
 * ---------------------------------------------------------------------------------------------- */

/* Creates a pool of `capacity` chunk slots (64 KiB of blocks + 1 KiB of heights each). */
hc_status hc_pool_create(hc_ctx *ctx, uint32_t capacity, hc_pool **out);
void hc_pool_destroy(hc_pool *pool);
uint32_t hc_pool_capacity(const hc_pool *pool);
/* Device base pointers of the pool (slot s at blocks + s*32768, heights + s*1024). */
hc_status hc_pool_buffers(const hc_pool *pool, uint16_t **blocks, int8_t **heights);
/* Copies `count` chunks into slots [first, first + count). `src_on_device` selects device or host
 * sources. Asynchronous on `stream`. */
hc_status hc_pool_upload(hc_pool *pool, uint32_t first, uint32_t count, const uint16_t *blocks, const int8_t *heights,
                         int src_on_device, void *stream);

/* Copies slots [first, first + count) back to host or device memory (dst_on_device). Synchronous. */
hc_status hc_pool_download(hc_pool *pool, uint32_t first, uint32_t count, uint16_t *blocks, int8_t *heights,
                           int dst_on_device, void *stream);

/* Arena that receives a batch's meshes (all pointers on the device). Chunk i of the batch gets
 * results[5*i .. 5*i+4] = {opaque quads, transparent quads, first mesh, mesh count, status}
 * (status 0 = ok, 1 = arena full, 2 = bad neighbour slot); its meshes are meshes[first ..
 * first + count), whose offsets index `vertices` / `indices`. The arena layout across chunks
 * depends on scheduling; each chunk's meshes are byte-identical to hc_mesh_chunk. */
typedef struct hc_batch_arena {
	uint64_t quad_capacity; /* vertices hold 4 * quad_capacity, indices 6 * quad_capacity */
	uint32_t mesh_capacity;
	uint32_t *vertices;
	uint16_t *indices;
	hc_mesh_desc *meshes;
	uint32_t *results;
} hc_batch_arena;

/* The renderer's hand-off records (client/include/client/ChunkMesh.hpp:12-18 and
 * client/include/client/mesh/MeshInfo.hpp:9-12): ChunkMeshInfo (40 bytes) and the
 * MeshInfo<ChunkMeshInfo> draw record (52 bytes) that WorldRenderer::PushChunkMesh builds for each
 * mesh (client/include/client/WorldRenderer.hpp:69-87): the AABB in world units as float, the
 * u32 AABB (1/16 voxel) divided by 16 plus the chunk's base position. */
typedef struct hc_chunk_mesh_info {
	float aabb_min[3], aabb_max[3];
	int32_t base_position[3]; /* chunk position * 32 */
	uint32_t transparent;
} hc_chunk_mesh_info;
typedef struct hc_mesh_info {
	uint32_t index_count, first_index, vertex_offset; /* into the arena's index and vertex buffers */
	hc_chunk_mesh_info info;
} hc_mesh_info;

/* Draw records for `n` mesh descriptors of an arena (device arrays): chunk i of the batch (the
 * descriptor's `chunk`) is at chunk_positions[3i .. 3i+2] (device int32). Asynchronous. */
hc_status hc_mesh_infos(hc_ctx *ctx, const hc_mesh_desc *meshes, uint32_t n, const int32_t *chunk_positions,
                        hc_mesh_info *out, void *stream);

typedef struct hc_batch_plan hc_batch_plan;

enum { HC_BATCH_PERSISTENT = 0, HC_BATCH_PER_CHUNK = 1, HC_BATCH_AUTO = 2 };
/* Persistent-form variants (see HC_BATCH_AUTO): the relight (a batch light pass or a window per
 * chunk), CTAs per chunk, chunks a CTA takes per claim of the work counter, and the emission
 * scheme (quad records past shared memory kept in a global scratch, or no scratch: the emission
 * merges the planes again in windows of records). */
enum {
	HC_VARIANT_LIGHT_PASS = 0, /* batch light pass, one CTA per chunk, 1 chunk per claim, record scratch */
	HC_VARIANT_WINDOW = 1,     /* each chunk relights its own 62^3 window, one CTA per chunk */
	HC_VARIANT_CLUSTER2 = 2,   /* window relight, two CTAs (a cluster) per chunk */
	HC_VARIANT_CLUSTER4 = 3,   /* window relight, four CTAs per chunk */
	HC_VARIANT_CLAIM2 = 4,     /* as HC_VARIANT_LIGHT_PASS, 2 chunks per claim */
	HC_VARIANT_CLAIM4 = 5,     /* as HC_VARIANT_LIGHT_PASS, 4 chunks per claim */
	HC_VARIANT_NO_SCRATCH = 6, /* as HC_VARIANT_LIGHT_PASS, quad records in shared memory only */
	HC_VARIANT_COUNT = 7
};
/* Mode that builds exactly one persistent variant (no timing), e.g. to profile the one an
 * HC_BATCH_AUTO plan chose: a profiler's per-launch cost distorts the autotuner's own timing. */
#define HC_BATCH_VARIANT(v) (16 + (v))

/* Plans meshing `n` chunks whose neighbour slot table (n x 27 int32, device) is `neighbours`:
 * mode HC_BATCH_PERSISTENT captures {plane refresh, batch light pass, persistent work-stealing
 * kernel} as a CUDA graph; HC_BATCH_PER_CHUNK launches the single-chunk kernel once per chunk;
 * HC_BATCH_AUTO is an autotuner: it captures every HC_VARIANT_* of the persistent form, times each
 * on this batch (its arena receives the output, identical for all) and keeps the fastest. Large
 * batches favour the light pass; a few heavy chunks favour clusters. `ctas_per_sm` (0 = automatic)
 * sizes the persistent grid. */
hc_status hc_batch_plan_create(hc_ctx *ctx, hc_pool *pool, const int32_t *neighbours, uint32_t n,
                               const hc_batch_arena *arena, int mode, int ctas_per_sm, hc_batch_plan **out);
void hc_batch_plan_destroy(hc_batch_plan *plan);
/* The persistent variant the plan runs and, after HC_BATCH_AUTO, the time each variant took on
 * the batch (ms per variant, HC_VARIANT_COUNT entries; 0 where not timed). */
hc_status hc_batch_plan_variant(const hc_batch_plan *plan, int *variant, float ms[HC_VARIANT_COUNT]);
/* Waits for the last launch and gives the device time of its stages (ms, CUDA events recorded
 * inside the plan): [0] bit-plane refresh, [1] batch light pass (0 for other variants), [2] the
 * meshing kernel(s). No counterpart in the reference (its runner is not staged). */
hc_status hc_batch_plan_stage_ms(hc_batch_plan *plan, float ms[3]);
/* Enqueues one run of the plan on `stream` (NULL = the context stream). */
hc_status hc_batch_plan_launch(hc_batch_plan *plan, void *stream);
/* Waits for the last launch and reads the arena cursors: quads and meshes written (or required,
 * when some chunk reported a full arena) and the number of chunks with a non-zero status. */
hc_status hc_batch_plan_result(hc_batch_plan *plan, uint64_t *quads, uint32_t *meshes, uint32_t *failed_chunks);
/* Copies the last run's output to host memory: the first `quads` quads of the arena (4 vertices
 * of 2 uint32 words and 6 uint16 indices each), `meshes` descriptors and the n x 5 result words.
 * Any destination may be NULL to skip it. Synchronous. */
hc_status hc_batch_plan_download(hc_batch_plan *plan, uint64_t quads, uint32_t meshes, uint32_t *vertices,
                                 uint16_t *indices, hc_mesh_desc *mesh_descs, uint32_t *results);
/* The same copies enqueued on `stream` (NULL = the stream of the last launch) without waiting:
 * with pinned destinations a client overlaps one batch's download with the next batch's upload
 * and meshing (two pools and plans in flight). No counterpart in the reference. */
hc_status hc_batch_plan_download_async(hc_batch_plan *plan, uint64_t quads, uint32_t meshes, uint32_t *vertices,
                                       uint16_t *indices, hc_mesh_desc *mesh_descs, uint32_t *results, void *stream);



/* ----------------------------------------------------------------------------------------------
 * Block edits on a resident world, then relight + remesh of the chunks they touch.
 *
 * Replaces the reference's edit task chain: ChunkTaskRunner<kSetBlock>::Run
 * (client/src/ChunkSetBlockTask.cpp:37-131), the sunlight-height recomputation of
 * ChunkTaskRunner<kFloodSunlight>::Run (client/src/ChunkFloodSunlightTask.cpp:33-66) and
 * ChunkTaskRunner<kSetSunlight>::Run (client/src/ChunkSetSunlightTask.cpp:28-90), followed by the
 * kMesh runs they trigger. A world is a dense grid of chunk positions over a pool.
 * ---------------------------------------------------------------------------------------------- */
typedef struct hc_world hc_world;
typedef struct hc_world_desc {
	int32_t nx, ny, nz;    /* grid size in chunks */
	int32_t cx0, cy0, cz0; /* chunk coordinate of grid cell (0, 0, 0) */
} hc_world_desc;
/* One edit: world voxel coordinates and the new raw block (low 16 bits of `block`). */
typedef struct hc_edit {
	int32_t x, y, z;
	uint32_t block;
} hc_edit;

/* Grid cell (ix, iy, iz), index ix + nx * (iz + nz * iy), holds chunk (cx0 + ix, cy0 + iy, cz0 + iz)
 * in pool slot slots[index] (host array), or -1 when that chunk is not resident. A resident
 * chunk's blocks and heights change only through the hc_world_* calls below, or the caller says
 * so with hc_world_touch. Calls on one world are ordered on the stream they name. */
hc_status hc_world_create(hc_ctx *ctx, hc_pool *pool, const hc_world_desc *desc, const int32_t *slots, hc_world **out);
void hc_world_destroy(hc_world *world);

/* Applies `n` edits in order (the last edit of a voxel wins; edits outside the resident world are
 * ignored), recomputes the sunlight heights of every edited column with the reference's rule
 * (a chunk's column is dark, 32, when the chunk above has a positive height there, else one above
 * its highest block that stops vertical light; the top grid layer counts as lit from above),
 * cascading down, and marks for remeshing every chunk whose light window holds a changed block
 * (ChunkShouldRemesh, client/include/client/ChunkMeshTask.inl:9-15) and the 27 chunks around
 * every chunk whose heights changed. `edits` is a host or device array (src_on_device). */
hc_status hc_world_apply_edits(hc_world *world, const hc_edit *edits, uint32_t n, int src_on_device, void *stream);

/* A chunk entering the world (replaces ChunkTaskRunner<kGenerate>::Run,
 * client/src/ChunkGenerateTask.cpp:21-40): its generated blocks (32768 uint16) and sunlight
 * heights (1024 int8), host memory, are copied into pool slot `slot`; then its stored edits are
 * applied in order, as the reference applies a ChunkEntry from its database: block entries in the
 * PackedChunkBlockEntry layout (uint32: cell index << 16 | raw block) and sunlight entries in the
 * PackedChunkSunlightEntry layout (uint16: column index << 6 | height)
 * (common/include/common/Data.hpp:36-86). The chunk is then marked for remeshing. */
typedef struct hc_chunk_load {
	int32_t cx, cy, cz; /* chunk position */
	int32_t slot;       /* free pool slot */
	const uint16_t *blocks;
	const int8_t *heights;
	const uint32_t *block_entries;   /* may be NULL when n_block_entries is 0 */
	const uint16_t *sunlight_entries;
	uint32_t n_block_entries, n_sunlight_entries;
} hc_chunk_load;

/* Loads `n` chunks (positions outside the grid are skipped). Each is marked for remeshing, and so
 * is every marked neighbour that waited for it. Returns once the host data has been copied. */
hc_status hc_world_load(hc_world *world, const hc_chunk_load *loads, uint32_t n, void *stream);
/* Takes `n` chunks (positions: host int32 x 3n) out of the world; their slots are free once the
 * stream passes this point. A pending remesh of them is dropped (ChunkTaskData<kMesh>::OnUnload). */
hc_status hc_world_unload(hc_world *world, const int32_t *positions, uint32_t n, void *stream);
/* How many CTAs (SMs) mesh one chunk together in hc_world_remesh: 1, 2, 4 (default) or 8. More
 * finish a pass of few heavy chunks sooner; 1 gives the most chunks per second on large passes. */
hc_status hc_world_set_cluster(hc_world *world, int ctas_per_chunk);
/* Rebuilds the per-chunk light planes of every resident chunk before the next remesh: call after
 * writing resident chunks' pool data by other means (hc_pool_upload). Synchronous. */
hc_status hc_world_touch(hc_world *world, void *stream);

/* Relights and meshes every marked chunk whose 26 neighbours are resident (the reference's kMesh
 * waits for them too), in grid order, into `arena` (chunk i of the batch = cells[i]; arena
 * results hold one entry per grid cell); clears their marks. A marked chunk with a missing
 * neighbour waits until a neighbour is loaded. cells (host, cap >= grid cells) receives the grid
 * indices; *n_remeshed their number. A chunk that does not fit the arena reports status 1 in its
 * result words, stays marked for the next remesh, and the call returns HC_ERR_CAPACITY. */
hc_status hc_world_remesh(hc_world *world, const hc_batch_arena *arena, int32_t *cells, uint32_t cap,
                          uint32_t *n_remeshed, uint64_t *quads, uint32_t *meshes, void *stream);

/* ----------------------------------------------------------------------------------------------
 * Request server: continuous batching of world requests into fixed ticks.
 *
 * Replaces the reference's chunk task scheduling: ChunkTaskPool (client/src/ChunkTaskPool.cpp:
 * 16-130) with its worker threads (client/src/WorldWorker.cpp:18-27) and LocalClient's chunk loader
 * (client/src/LocalClient.cpp:14-27). Requests arrive at any time (hc_server_submit); every tick
 * the server admits, in arrival order, the requests that fit the tick (edits, with a fill counted
 * as its voxels, up to max_edits_per_tick; loads up to max_loads_per_tick; unloads up to 4,096; a
 * load needs a free pool slot, and slots freed by unloads return once their tick completes) and runs
 * one device pass for them: unloads, loads, edits, sunlight heights, then relight + remesh of every
 * chunk they marked (as hc_world_*). Up to `depth` passes are in flight; each has its own arena.
 * A load or unload of a chunk that an earlier request of the same tick edits waits for the next
 * tick, so the result equals applying the requests one at a time in arrival order.
 * ---------------------------------------------------------------------------------------------- */
typedef struct hc_server hc_server;

typedef struct hc_server_config {
	uint32_t tick_us;            /* tick period in microseconds */
	uint32_t depth;              /* passes in flight, 1..8 */
	uint32_t max_edits_per_tick; /* edits per tick, a fill counting as its voxels */
	uint32_t max_loads_per_tick; /* loads per tick (a tick also takes up to 4,096 unloads) */
	uint64_t arena_quads;        /* per pass in flight; a chunk that does not fit is remeshed by a later pass */
	uint32_t arena_meshes;
	uint32_t ctas_per_chunk;     /* SMs meshing one chunk together (hc_world_set_cluster); 0: 4 */
} hc_server_config;

enum { HC_REQ_EDIT = 0, HC_REQ_FILL = 1, HC_REQ_LOAD = 2, HC_REQ_UNLOAD = 3 };

typedef struct hc_request {
	uint32_t kind;          /* HC_REQ_* */
	uint32_t block;         /* EDIT, FILL: new raw block */
	int32_t x, y, z;        /* EDIT: voxel; FILL: lowest corner voxel; LOAD, UNLOAD: chunk position */
	uint32_t size;          /* FILL: edge length in voxels, 1..32 */
	const uint16_t *blocks; /* LOAD: 32768 blocks (host), read when the request is admitted */
	const int8_t *heights;  /* LOAD: 1024 sunlight heights (host) */
	uint64_t tag;           /* echoed in the completion */
	const uint32_t *block_entries;    /* LOAD: stored edits, as in hc_chunk_load (host) */
	const uint16_t *sunlight_entries;
	uint32_t n_block_entries, n_sunlight_entries;
} hc_request;

typedef struct hc_completion {
	uint64_t tag;
	uint32_t kind;
	uint32_t status; /* 0 done; 1 rejected (position outside the grid, bad fill size, missing data) */
	uint64_t tick;
	uint64_t submit_ns, done_ns; /* steady clock: submitted, and its pass observed complete */
} hc_completion;

typedef struct hc_server_stats {
	uint64_t ticks, requests_done, requests_rejected;
	uint64_t chunks_remeshed, chunks_requeued, quads;
	uint64_t edits, loads, unloads;
	uint64_t gpu_ns_total, gpu_ns_max; /* device time of the passes */
	uint32_t pool_capacity, resident, free_slots, queued;
} hc_server_stats;

/* Called on the server's completion thread after each pass, with host copies of its output: the
 * remeshed grid cells, their result words (5 each), and the arena's vertices, indices, mesh
 * descriptors (offsets as in hc_batch_arena) and draw records. Every pass computes the draw
 * records on the device; the sink, for tests and tools, costs a full read-back. */
typedef void (*hc_tick_sink)(void *user, uint64_t tick, uint32_t n_chunks, const int32_t *cells,
                             const uint32_t *results, const uint32_t *vertices, const uint16_t *indices,
                             const hc_mesh_desc *meshes, const hc_mesh_info *infos, uint64_t quads,
                             uint32_t mesh_count);

/* Creates a server over an empty world grid with a chunk pool of `pool_capacity` slots (0: as many
 * as free device memory allows, keeping 2 GiB, at most 65536). */
hc_status hc_server_create(hc_ctx *ctx, const hc_world_desc *desc, uint32_t pool_capacity,
                           const hc_server_config *config, hc_server **out);
/* Stops the server (as hc_server_stop) and frees it. */
void hc_server_destroy(hc_server *server);
/* Queues requests (thread-safe). */
hc_status hc_server_submit(hc_server *server, const hc_request *requests, uint32_t n);
/* Starts the tick and completion threads. */
hc_status hc_server_start(hc_server *server);
/* Waits until every submitted request has completed and no chunk is left marked, then stops. */
hc_status hc_server_stop(hc_server *server);
/* Without the threads: admits what fits one tick, runs its pass and waits for it. */
hc_status hc_server_step(hc_server *server, uint32_t *admitted);
/* Takes up to `cap` completions, oldest first. */
hc_status hc_server_poll(hc_server *server, hc_completion *out, uint32_t cap, uint32_t *n);
hc_status hc_server_get_stats(hc_server *server, hc_server_stats *out);
/* Sets the per-pass sink (NULL: none); only while stopped. */
hc_status hc_server_set_sink(hc_server *server, hc_tick_sink sink, void *user);
/* The pool slot of every grid cell (-1: not resident) as of the last admitted tick. */
hc_status hc_server_resident(hc_server *server, int32_t *cell_slots);
/* The server's chunk pool (for hc_pool_download while it is idle). */
hc_pool *hc_server_pool(hc_server *server);
/* Replays a timed request trace on a started server: request i is submitted arrival_ns[i] after
 * the call starts (its tag becomes i); returns once all have completed, with latency_ns[i] from
 * its arrival time to its completion, ticks[i] the tick that admitted it (ticks may be NULL) and
 * *elapsed_ns from the start to the last completion. */
hc_status hc_server_replay(hc_server *server, const hc_request *requests, const uint64_t *arrival_ns, uint32_t n,
                           uint64_t *latency_ns, uint64_t *ticks, uint64_t *elapsed_ns);

/* ----------------------------------------------------------------------------------------------
 * Batched meshing that allocates nothing. No counterpart in the reference.
 *
 * For callers that cannot allocate device memory (a host application's frame loop under a fixed
 * device-memory budget, or a plugin whose host owns every allocation): the same batched kernel
 * and output as hc_batch_plan_launch, with every input and output buffer passed in by the caller
 * (chunk pool arrays, neighbour slot table, vertices, indices, mesh descriptors, all device
 * memory) and no context. Its scratch (arena cursors, work counter and the five result words per
 * chunk) and its block tables live in fixed device arrays of this library (about 390 KB per GPU,
 * held until exit). It calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * Limit: 1..HC_NOALLOC_MAX_CHUNKS chunks per call; larger batches return HC_ERR_CAPACITY.
 * Output buffers too small for the batch: HC_ERR_CAPACITY, with the required quad and mesh counts
 * written to *quads and *mesh_count (the chunks that did not fit have status 1 and no output).
 * The first call on a device (the current one) sets the tables up with synchronous copies; make
 * it before any stream capture. The set-up is kept for the life of the process: a device reset
 * (cudaDeviceReset) discards the tables, so do not call this entry point on a device again after
 * resetting it. All calls on a device share the scratch, so calls that overlap on the GPU race; run
 * them in one stream or one at a time. Synchronous: it waits for its stream.
 * results_host (n x 5 words, may be NULL) receives {opaque quads, transparent quads, first mesh,
 * mesh count, status} per chunk; error_text (may be NULL) receives a message.
 * ---------------------------------------------------------------------------------------------- */
#define HC_NOALLOC_MAX_CHUNKS 16384u
hc_status hc_mesh_batch_noalloc(const uint16_t *pool_blocks, const int8_t *pool_heights, uint32_t pool_capacity,
                                const int32_t *neighbours, uint32_t n, uint32_t *vertices, uint16_t *indices,
                                hc_mesh_desc *meshes, uint64_t quad_capacity, uint32_t mesh_capacity,
                                uint32_t *results_host, uint64_t *quads, uint32_t *mesh_count,
                                uint32_t *failed_chunks, void *stream, char *error_text, size_t error_text_size);

#ifdef __cplusplus
}
#endif

#endif /* HC_GB300_H */
