// Kernels and the C ABI of the GB300 chunk relighter + mesher (include/hc_gb300.h).
#include <cuda_runtime.h>

#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hc_gb300.h"
#include "hc_mesh.cuh"
#include "hc_world.cuh"
#include "hc_internal.h"
#include "hc_registry.h"

namespace hc {

struct Refs27 {
	const uint16_t *blk[27];
	const int8_t *hgt[27];
	const uint32_t *pln[27]; // null: seed the relight window from the blocks
};

__device__ __forceinline__ Smem &smem() {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	return *reinterpret_cast<Smem *>(smem_raw);
}

// One chunk, one CTA: the plain per-chunk form.
__global__ void __launch_bounds__(kThreads, 1) k_mesh_single(Refs27 refs, DevTables T, Arena A) {
	Smem &S = smem();
	if (threadIdx.x < 27) {
		S.blk[threadIdx.x] = refs.blk[threadIdx.x];
		S.hgt[threadIdx.x] = refs.hgt[threadIdx.x];
		S.pln[threadIdx.x] = refs.pln[threadIdx.x];
		S.lvl[threadIdx.x] = S.edg[threadIdx.x] = nullptr;
	}
	__syncthreads();
	mesh_chunk_cta(S, T, A, 0);
}

// Planes of the listed pool slots (grid-stride over slot x row).
__global__ void __launch_bounds__(256, 4) k_planes_pool(const uint16_t *pool_blocks, const int8_t *pool_heights,
                                                      const int32_t *slots, uint32_t n, DevTables T, uint32_t *planes) {
	__shared__ DevClass cls[256];
	for (int i = threadIdx.x; i < 256; i += blockDim.x)
		cls[i] = T.classes[i];
	__syncthreads();
	const uint64_t total = (uint64_t)n * kPlaneWords;
	for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x) {
		const uint32_t i = (uint32_t)(g / kPlaneWords), r = (uint32_t)(g % kPlaneWords);
		const size_t slot = (size_t)slots[i];
		planes_row(pool_blocks + slot * 32768, pool_heights + slot * 1024, cls, T.class_of, (int)r,
		           planes + slot * kPlaneStride);
	}
}

// Blank test of every chunk of a batch ahead of the mesher, one warp per chunk, from the layer
// summaries of the chunk and its six face neighbours (as stage_classes does at its start): the
// mesher then skips blank chunks without staging or prefetching them. A chunk with a bad
// neighbour slot is left to the mesher, which reports it.
__global__ void __launch_bounds__(256) k_blank_items(const uint32_t *planes, uint32_t pool_cap, const int32_t *nbr,
                                                     uint32_t n, uint8_t *blank) {
	const uint32_t i = blockIdx.x * 8 + (threadIdx.x >> 5);
	const int lane = threadIdx.x & 31;
	if (i >= n)
		return;
	const int32_t s = lane < 27 ? __ldg(nbr + (size_t)i * 27 + lane) : 0;
	const bool bad = __any_sync(0xffffffffu, lane < 27 && (s < 0 || (uint32_t)s >= pool_cap));
	const auto layers = [&](int k) { // lane's layer word of neighbour k
		const int32_t sk = __shfl_sync(0xffffffffu, s, k);
		return bad ? 0u : __ldg(planes + (size_t)sk * kPlaneStride + kPlaneLayerOff + lane);
	};
	const uint32_t mine = layers(26), xm = layers(nb_index(-1, 0, 0)), xp = layers(nb_index(kChunk, 0, 0));
	const uint32_t zm = layers(nb_index(0, 0, -1)), zp = layers(nb_index(0, 0, kChunk));
	const uint32_t ym = __shfl_sync(0xffffffffu, layers(nb_index(0, -1, 0)), 31);
	const uint32_t yp = __shfl_sync(0xffffffffu, layers(nb_index(0, kChunk, 0)), 0);
	const uint32_t open = (mine & kLayerOpen) | (xm & kLayerOpenX31) | (xp & kLayerOpenX0) | (zm & kLayerOpenZ31) |
	                      (zp & kLayerOpenZ0) | ((ym | yp) & kLayerOpen);
	const bool is_blank = !bad && (!__any_sync(0xffffffffu, mine & kLayerContent) || !__any_sync(0xffffffffu, open));
	if (lane == 0)
		blank[i] = is_blank;
}

// Planes of the 27 chunks of a single-chunk call.
__global__ void __launch_bounds__(256) k_planes_refs(Refs27 refs, DevTables T, uint32_t *planes) {
	__shared__ DevClass cls[256];
	for (int i = threadIdx.x; i < 256; i += blockDim.x)
		cls[i] = T.classes[i];
	__syncthreads();
	const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t i = g / kPlaneWords, r = g % kPlaneWords;
	if (i < 27)
		planes_row(refs.blk[i], refs.hgt[i], cls, T.class_of, (int)r, planes + (size_t)i * kPlaneStride);
}

// Relight only, writing the 34^3 region the mesher reads.
__global__ void __launch_bounds__(kThreads, 1) k_relight_single(Refs27 refs, DevTables T, uint8_t *light34) {
	Smem &S = smem();
	if (threadIdx.x < 27) {
		S.blk[threadIdx.x] = refs.blk[threadIdx.x];
		S.hgt[threadIdx.x] = refs.hgt[threadIdx.x];
		S.pln[threadIdx.x] = refs.pln[threadIdx.x];
		S.lvl[threadIdx.x] = S.edg[threadIdx.x] = nullptr;
	}
	for (int i = threadIdx.x; i < 256; i += kThreads)
		S.classes[i] = T.classes[i];
	__syncthreads();
	relight_window(S, T);
	__syncthreads();
	for (int i = threadIdx.x; i < kLtCells; i += kThreads)
		light34[i] = (uint8_t)(S.cell[i] & 0xffu);
}

enum : uint32_t { kChunkBadSlot = 2 };

// Points S.blk / S.hgt at the 27 neighbour slots of batch item `item`; false if a slot is invalid.
// With `levels` (the batch light pass), S.lvl / S.edg point at the 27 chunks' level planes and edge
// bits, found through the batch's own chunk numbering nbr_local.
__device__ bool load_refs(Smem &S, const uint16_t *pool_blocks, const int8_t *pool_heights, const uint32_t *pool_planes,
                          uint32_t pool_cap, const int32_t *nbr, uint32_t item, const uint32_t *levels = nullptr,
                          const uint32_t *edges = nullptr, const int32_t *nbr_local = nullptr,
                          const uint32_t *lflags = nullptr) {
	__shared__ int s_bad;
	if (threadIdx.x == 0)
		s_bad = 0;
	__syncthreads();
	if (threadIdx.x < 27) {
		const int32_t slot = nbr[(size_t)item * 27 + threadIdx.x];
		if (slot < 0 || (uint32_t)slot >= pool_cap) {
			s_bad = 1;
			S.blk[threadIdx.x] = pool_blocks;
			S.hgt[threadIdx.x] = pool_heights;
			S.pln[threadIdx.x] = nullptr;
			S.lvl[threadIdx.x] = S.edg[threadIdx.x] = nullptr;
		} else {
			S.blk[threadIdx.x] = pool_blocks + (size_t)slot * 32768;
			S.hgt[threadIdx.x] = pool_heights + (size_t)slot * 1024;
			S.pln[threadIdx.x] = pool_planes ? pool_planes + (size_t)slot * kPlaneStride : nullptr;
			const size_t loc = levels ? (size_t)nbr_local[(size_t)item * 27 + threadIdx.x] : 0;
			S.lvl[threadIdx.x] = levels ? levels + loc * kLevelSlotWords : nullptr;
			S.edg[threadIdx.x] = levels ? edges + loc * kEdgeSlotWords : nullptr;
			S.lfl[threadIdx.x][0] = lflags ? __ldg(lflags + 2 * loc) : 0u;
			S.lfl[threadIdx.x][1] = lflags ? __ldg(lflags + 2 * loc + 1) : 0u;
		}
	}
	__syncthreads();
	return s_bad == 0;
}

__device__ void bad_item(const Arena &A, uint32_t item, unsigned int *failed) {
	if (threadIdx.x == 0) {
		uint32_t *r = A.results + 5 * (size_t)item;
		r[0] = r[1] = r[2] = r[3] = 0;
		r[4] = kChunkBadSlot;
		atomicAdd(failed, 1u);
	}
}

// Starts an asynchronous copy of [p, p + bytes) into L2 (bytes a multiple of 16, p 16-byte aligned).
__device__ __forceinline__ void prefetch_l2(const void *p, uint32_t bytes) {
	asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Prefetches what the next chunk of a batch reads first. With the batch light pass the chunk reads
// its own opaque/blank planes and layer words, its class ids and its light levels (the neighbours
// only at the apron); with a window relight, the bit planes of all 27 chunks and its class ids;
// without planes, its blocks.
__device__ __forceinline__ void prefetch_item(const uint16_t *pool_blocks, const uint32_t *pool_planes, uint32_t pool_cap,
                                              const int32_t *nbr, uint32_t item, const uint32_t *levels,
                                              const int32_t *nbr_local) {
	const int t = threadIdx.x;
	if (t < 27) {
		const int32_t slot = nbr[(size_t)item * 27 + t];
		if (slot >= 0 && (uint32_t)slot < pool_cap) {
			const uint32_t *P = pool_planes + (size_t)slot * kPlaneStride;
			if (pool_planes && levels) {
				if (t == 26) {
					prefetch_l2(P + kPlaneOpaque * kPlaneWords, (kPlaneClassOff - kPlaneOpaque * kPlaneWords) * sizeof(uint32_t));
					prefetch_l2(P + kPlaneClassOff, 32768);
					const size_t loc = (size_t)nbr_local[(size_t)item * 27 + 26];
					prefetch_l2(levels + loc * kLevelSlotWords, (uint32_t)(kLevelSlotWords * sizeof(uint32_t)));
				}
			} else if (pool_planes) {
				prefetch_l2(P, kPlaneBits * sizeof(uint32_t));
				if (t == 26)
					prefetch_l2(P + kPlaneClassOff, 32768);
			} else if (t == 26) {
				for (int q = 0; q < 4; ++q)
					prefetch_l2(pool_blocks + (size_t)slot * 32768 + q * 8192, 16384);
			}
		}
	}
}

// Batched form: a persistent grid; each CTA takes chunks from a device work counter, claiming the
// next one while it meshes the current one so that the next chunk's data is already in L2.
__global__ void __launch_bounds__(kThreads, 1)
    k_mesh_batch(const uint16_t *pool_blocks, const int8_t *pool_heights, const uint32_t *pool_planes, uint32_t pool_cap,
                 const int32_t *nbr, uint32_t n, const uint32_t *n_dev, unsigned int *work, unsigned int *failed,
                 DevTables T, Arena A, const uint32_t *levels, const uint32_t *edges, const int32_t *nbr_local,
                 const uint32_t *lflags, const uint8_t *item_blank, uint32_t claim) {
	Smem &S = smem();
	__shared__ uint32_t s_next;
	if (n_dev) // the batch length is known on the device only (a world remesh)
		n = *n_dev;
	if (threadIdx.x == 0)
		s_next = atomicAdd(work, claim);
	__syncthreads();
	uint32_t item = s_next, left = claim; // a claim takes `claim` consecutive chunks
	for (;;) {
		if (item >= n)
			break;
		__syncthreads(); // everyone has read s_next
		uint32_t next = item + 1;
		if (left == 1) {
			if (threadIdx.x == 0)
				s_next = atomicAdd(work, claim);
			__syncthreads();
			next = s_next;
		}
		if (next < n && !(item_blank && item_blank[next]))
			prefetch_item(pool_blocks, pool_planes, pool_cap, nbr, next, levels, nbr_local);
		if (item_blank && item_blank[item]) { // no quad: the results a blank chunk gets
			if (threadIdx.x < 5)
				A.results[5 * (size_t)item + threadIdx.x] = threadIdx.x == 4 ? kChunkOk : 0u;
		} else if (load_refs(S, pool_blocks, pool_heights, pool_planes, pool_cap, nbr, item, levels, edges, nbr_local,
		                     lflags)) {
			mesh_chunk_cta(S, T, A, item);
			if (threadIdx.x == 0 && A.results[5 * (size_t)item + 4] != kChunkOk)
				atomicAdd(failed, 1u);
		} else {
			bad_item(A, item, failed);
		}
		__syncthreads();
		left = left == 1 ? claim : left - 1;
		item = next;
	}
}

// Batched form for latency: clusters of `csize` CTAs take chunks from the work counter and mesh
// each chunk together (mesh_chunk_cta with a Split), so a pass of few heavy chunks finishes sooner.
__global__ void __launch_bounds__(kThreads, 1)
    k_mesh_cluster(const uint16_t *pool_blocks, const int8_t *pool_heights, const uint32_t *pool_planes,
                   uint32_t pool_cap, const int32_t *nbr, uint32_t n, const uint32_t *n_dev, unsigned int *work,
                   unsigned int *failed, DevTables T, Arena A, const uint32_t *levels, const uint32_t *edges,
                   const int32_t *nbr_local, int csize) {
	namespace cg = cooperative_groups;
	cg::cluster_group cl = cg::this_cluster();
	const int rank = (int)cl.block_rank();
	Smem &S = smem();
	__shared__ uint32_t s_item;
	if (n_dev)
		n = *n_dev;
	for (;;) {
		if (rank == 0 && threadIdx.x == 0)
			s_item = atomicAdd(work, 1u);
		cl.sync();
		const uint32_t item = *cl.map_shared_rank(&s_item, 0);
		cl.sync(); // every CTA has read CTA 0's s_item: CTA 0 may now exit, or claim the next chunk
		if (item >= n)
			break;
		if (load_refs(S, pool_blocks, pool_heights, pool_planes, pool_cap, nbr, item, levels, edges, nbr_local)) {
			mesh_chunk_cta(S, T, A, item, Split{csize, rank});
			if (rank == 0 && threadIdx.x == 0 && A.results[5 * (size_t)item + 4] != kChunkOk)
				atomicAdd(failed, 1u);
		} else if (rank == 0) {
			bad_item(A, item, failed);
		}
		cl.sync(); // every CTA has read s_item and finished with the others' shared memory
	}
}

// Draw records of mesh descriptors (WorldRenderer::PushChunkMesh, WorldRenderer.hpp:69-87): the
// float AABB is the u32 one in 1/16 voxel divided by 16, plus the chunk's base position.
__global__ void k_mesh_infos(const hc_mesh_desc *meshes, uint32_t n, const int32_t *pos, hc_mesh_info *out) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const hc_mesh_desc d = meshes[i];
	hc_mesh_info m;
	m.index_count = d.index_count;
	m.first_index = d.index_offset;
	m.vertex_offset = d.vertex_offset;
	for (int c = 0; c < 3; ++c) {
		const int32_t base = pos[3 * (size_t)d.chunk + c] * 32;
		m.info.base_position[c] = base;
		m.info.aabb_min[c] = __fadd_rn(__fdiv_rn((float)d.aabb_min[c], 16.0f), (float)base);
		m.info.aabb_max[c] = __fadd_rn(__fdiv_rn((float)d.aabb_max[c], 16.0f), (float)base);
	}
	m.info.transparent = d.transparent;
	out[i] = m;
}

// The same with the number of descriptors in device memory (an arena's mesh cursor, capped).
__global__ void k_mesh_infos_dev(const hc_mesh_desc *meshes, const unsigned int *n_dev, uint32_t cap, const int32_t *pos,
                                 hc_mesh_info *out) {
	const uint32_t n = min(*n_dev, cap);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const hc_mesh_desc d = meshes[i];
		hc_mesh_info m;
		m.index_count = d.index_count;
		m.first_index = d.index_offset;
		m.vertex_offset = d.vertex_offset;
		for (int c = 0; c < 3; ++c) {
			const int32_t base = pos[3 * (size_t)d.chunk + c] * 32;
			m.info.base_position[c] = base;
			m.info.aabb_min[c] = __fadd_rn(__fdiv_rn((float)d.aabb_min[c], 16.0f), (float)base);
			m.info.aabb_max[c] = __fadd_rn(__fdiv_rn((float)d.aabb_max[c], 16.0f), (float)base);
		}
		m.info.transparent = d.transparent;
		out[i] = m;
	}
}

// Chunk positions of a world remesh list (for its draw records).
__global__ void k_remesh_positions(WorldDev W, const int32_t *list, const uint32_t *n, int32_t *pos) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= *n)
		return;
	int ix, iy, iz;
	cell_xyz(W, list[i], ix, iy, iz);
	pos[3 * i] = W.cx0 + ix, pos[3 * i + 1] = W.cy0 + iy, pos[3 * i + 2] = W.cz0 + iz;
}

// Plain form at scale: one launch per chunk.
__global__ void __launch_bounds__(kThreads, 1)
    k_mesh_item(const uint16_t *pool_blocks, const int8_t *pool_heights, const uint32_t *pool_planes, uint32_t pool_cap,
                const int32_t *nbr, uint32_t item, unsigned int *failed, DevTables T, Arena A) {
	Smem &S = smem();
	if (load_refs(S, pool_blocks, pool_heights, pool_planes, pool_cap, nbr, item)) {
		mesh_chunk_cta(S, T, A, item);
		if (threadIdx.x == 0 && A.results[5 * (size_t)item + 4] != kChunkOk)
			atomicAdd(failed, 1u);
	} else {
		bad_item(A, item, failed);
	}
}

} // namespace hc

using namespace hc;

struct hc_pool {
	hc_ctx *ctx = nullptr;
	uint32_t capacity = 0;
	uint16_t *d_blocks = nullptr;
	int8_t *d_heights = nullptr;
	uint32_t *d_planes = nullptr; // per-slot bit planes, refreshed by every batch run for its slots
};

struct hc_batch_plan {
	hc_ctx *ctx = nullptr;
	hc_pool *pool = nullptr;
	const int32_t *nbr = nullptr;
	uint32_t n = 0;
	hc_batch_arena arena{};
	int mode = HC_BATCH_PERSISTENT;
	int grid = 0;
	int variant = HC_VARIANT_LIGHT_PASS;
	float variant_ms[HC_VARIANT_COUNT] = {};
	int cluster_grid[HC_VARIANT_COUNT] = {}; // persistent grid of the cluster variants
	int32_t *d_slots = nullptr;            // distinct valid slots the batch reads (their planes are refreshed)
	uint32_t n_slots = 0;
	// batch light pass (persistent form): the distinct slots are the batch's chunks 0..n_slots-1
	int32_t *d_nb6 = nullptr;       // per batch chunk: its six face neighbours in the batch, or -1
	int32_t *d_nbr_local = nullptr; // n x 27: the neighbour table in batch chunk numbers
	uint8_t *d_blank = nullptr;     // per chunk to mesh: blank (no quad), from the layer summaries
	uint32_t *d_levels = nullptr;   // per batch chunk: 2 channels x 15 level planes
	uint32_t *d_edges = nullptr;    // per batch chunk: their x = 0 and x = 31 bits
	uint32_t *d_lflags = nullptr;   // per batch chunk and channel: which level planes are uniform
	unsigned long long *d_state = nullptr; // quad cursor, mesh cursor, work counter, failed chunks
	unsigned long long *h_state = nullptr; // pinned
	uint2 *d_spill = nullptr;              // quad records past the shared buffer, per CTA of any grid
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	cudaStream_t capture_stream = nullptr;
	cudaStream_t last = nullptr;
	// recorded around the stages of every run (event nodes of the graph): start, planes refreshed,
	// light pass done, meshes done
	cudaEvent_t stage_ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

struct hc_ctx {
	int device = 0;
	cudaStream_t stream = nullptr;
	uint8_t *d_class_of = nullptr;
	DevClass *d_classes = nullptr;
	// single-chunk staging and output
	uint16_t *d_blocks = nullptr;
	int8_t *d_heights = nullptr;
	uint16_t *h_blocks = nullptr; // pinned
	int8_t *h_heights = nullptr;  // pinned
	uint2 *d_verts = nullptr;
	uint16_t *d_idx = nullptr;
	hc_mesh_desc *d_meshes = nullptr;
	uint32_t *d_planes = nullptr;           // bit planes of the 27 chunks of a single-chunk call
	unsigned long long *d_cursor = nullptr; // [0] quads, [1] meshes (as unsigned int in the low word)
	uint32_t *d_results = nullptr;
	uint2 *d_spill = nullptr; // quad records past the shared buffer, one CTA
	uint32_t *h_results = nullptr; // pinned, 8 words
	size_t smem_bytes = 0;
	std::string err;
};

namespace {

hc_status fail(hc_ctx *ctx, hc_status s, const std::string &msg) {
	if (ctx)
		ctx->err = msg;
	return s;
}

#define HC_CUDA(ctx, call)                                                                                                 \
	do {                                                                                                                   \
		cudaError_t e_ = (call);                                                                                           \
		if (e_ != cudaSuccess)                                                                                             \
			return fail(ctx, e_ == cudaErrorMemoryAllocation ? HC_ERR_OUT_OF_MEMORY : HC_ERR_CUDA,                         \
			            std::string(#call) + ": " + cudaGetErrorString(e_));                                               \
	} while (0)

// The device row of one raw block value: face textures, light-pass and shape flags, tag, light level
// and custom-mesh fields.
DevClass class_row(const hc_block_props &p) {
	DevClass d;
	std::memset(&d, 0, sizeof(d));
	bool all_empty = true, all_opaque = true;
	for (int f = 0; f < 6; ++f) {
		d.tex[f] = p.tex[f];
		const bool empty = (p.tex[f] & 0x1fffu) == 0;
		all_empty &= empty;
		all_opaque &= !empty && !hc_tex_is_transparent(p.tex[f]);
	}
	const bool vertical = p.transparency == HC_TRANSPARENT;
	uint8_t flags = 0;
	if (p.transparency != HC_OPAQUE)
		flags |= kFIndirect;
	if (vertical || p.collision != HC_COLLISION_SOLID)
		flags |= kFDirect;
	if (vertical)
		flags |= kFVertical;
	if (p.mesh_kind == HC_MESH_NONE && all_opaque)
		flags |= kFOpaqueCube;
	if (p.mesh_kind == HC_MESH_NONE && all_empty)
		flags |= kFEmpty;
	const uint8_t tag = p.id == HC_BLK_AIR             ? kTagAir
	                    : p.id == HC_BLK_WATER         ? kTagSource
	                    : p.id == HC_BLK_FLOWING_WATER ? kTagFlow
	                                                   : kTagOther;
	d.flags = (uint8_t)(flags | (tag << kFTagShift));
	d.light = p.light_level;
	d.mesh_first = p.mesh_kind == HC_MESH_STATIC ? p.mesh_first : 0;
	const uint8_t param = p.mesh_kind == HC_MESH_STATIC ? p.mesh_count : (p.mesh_kind == HC_MESH_FLOW ? p.flow_variant : 0);
	d.mesh_meta = (uint8_t)(p.mesh_kind | (param << 2));
	return d;
}

// Derives the block classes from the registry: each distinct device row gets one id, in order of
// first appearance within its light-pass group (bit 7 indirect pass, bit 6 direct pass, 64 ids per
// group). Unused ids repeat the row of raw value 0. Uses no heap, so the context tables and the
// no-alloc entry point's static tables come from this one routine. False: more than 64 distinct
// rows in a group.
bool assign_classes(const hc_registry &reg, uint8_t *class_of, DevClass *classes) {
	uint32_t count[4] = {0, 0, 0, 0};
	bool used[256] = {false};
	for (uint32_t raw = 0; raw < 65536u; ++raw) {
		const DevClass d = class_row(reg.props[raw]);
		const uint32_t group = ((d.flags & kFIndirect) ? 2u : 0u) | ((d.flags & kFDirect) ? 1u : 0u);
		uint32_t c = 0;
		while (c < count[group] && std::memcmp(&classes[(group << 6) | c], &d, sizeof(d)) != 0)
			++c;
		if (c == count[group]) {
			if (c == 64)
				return false;
			classes[(group << 6) | c] = d;
			used[(group << 6) | c] = true;
			++count[group];
		}
		class_of[raw] = (uint8_t)((group << 6) | c);
	}
	for (uint32_t c = 0; c < 256; ++c)
		if (!used[c])
			classes[c] = classes[class_of[0]];
	return true;
}

bool build_classes(const hc_registry &reg, std::vector<uint8_t> &class_of, std::vector<DevClass> &classes) {
	class_of.assign(65536, 0);
	classes.assign(256, DevClass{});
	return assign_classes(reg, class_of.data(), classes.data());
}

hc_status upload_tables(hc_ctx *ctx) {
	static hc_registry reg; // 1.3 MB; built once per process
	static bool built = false;
	if (!built) {
		hc_registry_build(&reg);
		built = true;
	}
	std::vector<uint8_t> class_of;
	std::vector<DevClass> classes;
	if (!build_classes(reg, class_of, classes))
		return fail(ctx, HC_ERR_INVALID_ARG, "more than 256 distinct block classes");
	if (reg.static_face_count > HC_MAX_STATIC_FACES / 4)
		return fail(ctx, HC_ERR_INVALID_ARG, "too many static custom-mesh faces");
	uint64_t tt = 0, tl = 0, tp = 0;
	for (int t = 0; t < HC_TEX_COUNT; ++t) {
		tt |= (uint64_t)hc_tex_is_transparent((uint16_t)t) << t;
		tl |= (uint64_t)hc_tex_is_liquid((uint16_t)t) << t;
		tp |= (uint64_t)hc_tex_use_transparent_pass((uint16_t)t) << t;
	}
	HC_CUDA(ctx, cudaMalloc(&ctx->d_class_of, 65536));
	HC_CUDA(ctx, cudaMalloc(&ctx->d_classes, 256 * sizeof(DevClass)));
	HC_CUDA(ctx, cudaMemcpy(ctx->d_class_of, class_of.data(), 65536, cudaMemcpyHostToDevice));
	HC_CUDA(ctx, cudaMemcpy(ctx->d_classes, classes.data(), 256 * sizeof(DevClass), cudaMemcpyHostToDevice));
	HC_CUDA(ctx, cudaMemcpyToSymbol(c_tex_transparent, &tt, sizeof(tt)));
	HC_CUDA(ctx, cudaMemcpyToSymbol(c_tex_liquid, &tl, sizeof(tl)));
	HC_CUDA(ctx, cudaMemcpyToSymbol(c_tex_transpass, &tp, sizeof(tp)));
	HC_CUDA(ctx, cudaMemcpyToSymbol(c_static_faces, reg.static_faces, sizeof(hc_mesh_face) * reg.static_face_count));
	return HC_OK;
}

DevTables tables(const hc_ctx *ctx) { return DevTables{ctx->d_class_of, ctx->d_classes}; }

hc_status check_refs(hc_ctx *ctx, const uint16_t *const blocks[27], const int8_t *const heights[27],
                     bool device_pointers = false) {
	if (!blocks || !heights)
		return fail(ctx, HC_ERR_INVALID_ARG, "null neighbour array");
	for (int i = 0; i < 27; ++i) {
		if (!blocks[i] || !heights[i])
			return fail(ctx, HC_ERR_INVALID_ARG, "null chunk pointer at neighbour " + std::to_string(i));
		if (device_pointers && ((reinterpret_cast<uintptr_t>(blocks[i]) | reinterpret_cast<uintptr_t>(heights[i])) & 15u))
			return fail(ctx, HC_ERR_INVALID_ARG, "chunk arrays must be 16-byte aligned (neighbour " + std::to_string(i) + ")");
	}
	return HC_OK;
}

// Computes the bit planes of the 27 chunks into the context and points refs at them.
hc_status planes_for_refs(hc_ctx *ctx, Refs27 &refs, cudaStream_t st) {
	for (int i = 0; i < 27; ++i)
		refs.pln[i] = ctx->d_planes + (size_t)i * kPlaneStride;
	k_planes_refs<<<27 * kPlaneWords / 256, 256, 0, st>>>(refs, tables(ctx), ctx->d_planes);
	HC_CUDA(ctx, cudaGetLastError());
	return HC_OK;
}

// Runs the single-chunk kernel into the given device buffers; reads back the 5 result words.
hc_status run_single(hc_ctx *ctx, const Refs27 &refs, uint2 *verts, uint16_t *idx, hc_mesh_desc *meshes,
                     unsigned long long quad_cap, unsigned int mesh_cap, cudaStream_t st) {
	HC_CUDA(ctx, cudaMemsetAsync(ctx->d_cursor, 0, 2 * sizeof(unsigned long long), st));
	Arena A{verts, idx, meshes, ctx->d_cursor, reinterpret_cast<unsigned int *>(ctx->d_cursor + 1), quad_cap, mesh_cap,
	        ctx->d_results, ctx->d_spill};
	Refs27 r = refs;
	hc_status s = planes_for_refs(ctx, r, st);
	if (s != HC_OK)
		return s;
	k_mesh_single<<<1, kThreads, ctx->smem_bytes, st>>>(r, tables(ctx), A);
	HC_CUDA(ctx, cudaGetLastError());
	HC_CUDA(ctx, cudaMemcpyAsync(ctx->h_results, ctx->d_results, 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	HC_CUDA(ctx, cudaStreamSynchronize(st));
	return HC_OK;
}

} // namespace

extern "C" {

const char *hc_status_string(hc_status s) {
	switch (s) {
	case HC_OK:
		return "ok";
	case HC_ERR_INVALID_ARG:
		return "invalid argument";
	case HC_ERR_OUT_OF_MEMORY:
		return "out of memory";
	case HC_ERR_CAPACITY:
		return "output capacity exceeded";
	case HC_ERR_DEVICE_TIMEOUT:
		return "device wait timed out";
	case HC_ERR_CUDA:
		return "CUDA error";
	case HC_ERR_NO_DEVICE:
		return "no usable device";
	}
	return "unknown status";
}

const char *hc_last_error(const hc_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

hc_status hc_ctx_create(int device, hc_ctx **out) {
	if (!out)
		return HC_ERR_INVALID_ARG;
	*out = nullptr;
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
		return HC_ERR_NO_DEVICE;
	hc_ctx *ctx = new hc_ctx();
	ctx->device = device;
	hc_status s = HC_OK;
	do {
		if (cudaSetDevice(device) != cudaSuccess) {
			s = fail(ctx, HC_ERR_NO_DEVICE, "cudaSetDevice failed");
			break;
		}
		cudaDeviceProp prop;
		if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major < 10) {
			s = fail(ctx, HC_ERR_NO_DEVICE, "device is not a Blackwell-class GPU");
			break;
		}
		ctx->smem_bytes = sizeof(Smem);
		if (cudaFuncSetAttribute(k_mesh_single, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->smem_bytes) !=
		        cudaSuccess ||
		    cudaFuncSetAttribute(k_relight_single, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->smem_bytes) !=
		        cudaSuccess ||
		    cudaFuncSetAttribute(k_mesh_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->smem_bytes) !=
		        cudaSuccess ||
		    cudaFuncSetAttribute(k_mesh_item, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->smem_bytes) !=
		        cudaSuccess ||
		    cudaFuncSetAttribute(k_mesh_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->smem_bytes) !=
		        cudaSuccess) {
			s = fail(ctx, HC_ERR_NO_DEVICE, "cannot reserve " + std::to_string(ctx->smem_bytes) + " B of shared memory");
			break;
		}
		if ((s = upload_tables(ctx)) != HC_OK)
			break;
		const auto chk = [&](cudaError_t e, const char *what) {
			if (e != cudaSuccess && s == HC_OK)
				s = fail(ctx, e == cudaErrorMemoryAllocation ? HC_ERR_OUT_OF_MEMORY : HC_ERR_CUDA,
				         std::string(what) + ": " + cudaGetErrorString(e));
		};
		chk(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream");
		chk(cudaMalloc(&ctx->d_blocks, 27 * 32768 * sizeof(uint16_t)), "blocks");
		chk(cudaMalloc(&ctx->d_heights, 27 * 1024), "heights");
		chk(cudaMallocHost(&ctx->h_blocks, 27 * 32768 * sizeof(uint16_t)), "pinned blocks");
		chk(cudaMallocHost(&ctx->h_heights, 27 * 1024), "pinned heights");
		chk(cudaMalloc(&ctx->d_verts, (size_t)HC_CHUNK_MAX_QUADS * 4 * sizeof(uint2)), "vertices");
		chk(cudaMalloc(&ctx->d_idx, (size_t)HC_CHUNK_MAX_QUADS * 6 * sizeof(uint16_t)), "indices");
		chk(cudaMalloc(&ctx->d_meshes, HC_CHUNK_MAX_MESHES * sizeof(hc_mesh_desc)), "meshes");
		chk(cudaMalloc(&ctx->d_planes, 27 * (size_t)kPlaneStride * sizeof(uint32_t)), "planes");
		chk(cudaMalloc(&ctx->d_cursor, 2 * sizeof(unsigned long long)), "cursor");
		chk(cudaMalloc(&ctx->d_results, 8 * sizeof(uint32_t)), "results");
		chk(cudaMalloc(&ctx->d_spill, (size_t)kSpillRecs * sizeof(uint2)), "record scratch");
		chk(cudaMallocHost(&ctx->h_results, 8 * sizeof(uint32_t)), "pinned results");
	} while (0);
	if (s != HC_OK) {
		std::fprintf(stderr, "hc_ctx_create: %s\n", ctx->err.c_str());
		hc_ctx_destroy(ctx);
		return s;
	}
	*out = ctx;
	return HC_OK;
}

void hc_ctx_destroy(hc_ctx *ctx) {
	if (!ctx)
		return;
	cudaSetDevice(ctx->device);
	cudaFree(ctx->d_class_of);
	cudaFree(ctx->d_classes);
	cudaFree(ctx->d_blocks);
	cudaFree(ctx->d_heights);
	cudaFreeHost(ctx->h_blocks);
	cudaFreeHost(ctx->h_heights);
	cudaFree(ctx->d_verts);
	cudaFree(ctx->d_idx);
	cudaFree(ctx->d_meshes);
	cudaFree(ctx->d_planes);
	cudaFree(ctx->d_cursor);
	cudaFree(ctx->d_results);
	cudaFree(ctx->d_spill);
	cudaFreeHost(ctx->h_results);
	if (ctx->stream)
		cudaStreamDestroy(ctx->stream);
	delete ctx;
}

hc_status hc_mesh_chunk(hc_ctx *ctx, const uint16_t *const blocks[27], const int8_t *const heights[27], hc_chunk_mesh *out,
                        void *stream) {
	if (!ctx || !out)
		return HC_ERR_INVALID_ARG;
	hc_status s = check_refs(ctx, blocks, heights);
	if (s != HC_OK)
		return s;
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	for (int i = 0; i < 27; ++i) {
		std::memcpy(ctx->h_blocks + (size_t)i * 32768, blocks[i], 32768 * sizeof(uint16_t));
		std::memcpy(ctx->h_heights + (size_t)i * 1024, heights[i], 1024);
	}
	HC_CUDA(ctx, cudaMemcpyAsync(ctx->d_blocks, ctx->h_blocks, 27 * 32768 * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
	HC_CUDA(ctx, cudaMemcpyAsync(ctx->d_heights, ctx->h_heights, 27 * 1024, cudaMemcpyHostToDevice, st));
	Refs27 refs;
	for (int i = 0; i < 27; ++i) {
		refs.blk[i] = ctx->d_blocks + (size_t)i * 32768;
		refs.hgt[i] = ctx->d_heights + (size_t)i * 1024;
	}
	if ((s = run_single(ctx, refs, ctx->d_verts, ctx->d_idx, ctx->d_meshes, HC_CHUNK_MAX_QUADS, HC_CHUNK_MAX_MESHES, st)) !=
	    HC_OK)
		return s;
	const uint32_t *r = ctx->h_results;
	const uint32_t q = r[0] + r[1];
	out->mesh_count = r[3];
	out->vertex_count = 4 * q;
	out->index_count = 6 * q;
	if (r[4] != kChunkOk)
		return fail(ctx, HC_ERR_CAPACITY, "chunk exceeds the single-chunk output buffers");
	if (out->mesh_count > out->mesh_capacity || out->vertex_count > out->vertex_capacity ||
	    out->index_count > out->index_capacity)
		return fail(ctx, HC_ERR_CAPACITY, "caller output buffers too small");
	if (out->mesh_count && (!out->meshes || !out->vertices || !out->indices))
		return fail(ctx, HC_ERR_INVALID_ARG, "null output buffer");
	if (out->mesh_count) {
		HC_CUDA(ctx, cudaMemcpyAsync(out->meshes, ctx->d_meshes, out->mesh_count * sizeof(hc_mesh_desc),
		                             cudaMemcpyDeviceToHost, st));
		HC_CUDA(ctx, cudaMemcpyAsync(out->vertices, ctx->d_verts, (size_t)out->vertex_count * sizeof(uint2),
		                             cudaMemcpyDeviceToHost, st));
		HC_CUDA(ctx, cudaMemcpyAsync(out->indices, ctx->d_idx, (size_t)out->index_count * sizeof(uint16_t),
		                             cudaMemcpyDeviceToHost, st));
		HC_CUDA(ctx, cudaStreamSynchronize(st));
	}
	return HC_OK;
}

hc_status hc_mesh_chunk_device(hc_ctx *ctx, const uint16_t *const blocks[27], const int8_t *const heights[27],
                               hc_chunk_mesh *out, void *stream) {
	if (!ctx || !out)
		return HC_ERR_INVALID_ARG;
	hc_status s = check_refs(ctx, blocks, heights, true);
	if (s != HC_OK)
		return s;
	if (!out->meshes || !out->vertices || !out->indices)
		return fail(ctx, HC_ERR_INVALID_ARG, "null output buffer");
	if ((reinterpret_cast<uintptr_t>(out->vertices) & 15u) || (reinterpret_cast<uintptr_t>(out->indices) & 3u))
		return fail(ctx, HC_ERR_INVALID_ARG, "vertices must be 16-byte and indices 4-byte aligned");
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	Refs27 refs;
	for (int i = 0; i < 27; ++i) {
		refs.blk[i] = blocks[i];
		refs.hgt[i] = heights[i];
	}
	const unsigned long long qcap = std::min(out->vertex_capacity / 4, out->index_capacity / 6);
	if ((s = run_single(ctx, refs, reinterpret_cast<uint2 *>(out->vertices), out->indices, out->meshes, qcap,
	                    out->mesh_capacity, st)) != HC_OK)
		return s;
	const uint32_t *r = ctx->h_results;
	const uint32_t q = r[0] + r[1];
	out->mesh_count = r[3];
	out->vertex_count = 4 * q;
	out->index_count = 6 * q;
	if (r[4] != kChunkOk)
		return fail(ctx, HC_ERR_CAPACITY, "caller output buffers too small");
	return HC_OK;
}

hc_status hc_relight_chunk_device(hc_ctx *ctx, const uint16_t *const blocks[27], const int8_t *const heights[27],
                                  uint8_t *light34, void *stream) {
	if (!ctx || !light34)
		return HC_ERR_INVALID_ARG;
	hc_status s = check_refs(ctx, blocks, heights, true);
	if (s != HC_OK)
		return s;
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	Refs27 refs;
	for (int i = 0; i < 27; ++i) {
		refs.blk[i] = blocks[i];
		refs.hgt[i] = heights[i];
	}
	if ((s = planes_for_refs(ctx, refs, st)) != HC_OK)
		return s;
	k_relight_single<<<1, kThreads, ctx->smem_bytes, st>>>(refs, tables(ctx), light34);
	HC_CUDA(ctx, cudaGetLastError());
	HC_CUDA(ctx, cudaStreamSynchronize(st));
	return HC_OK;
}

hc_status hc_mesh_infos(hc_ctx *ctx, const hc_mesh_desc *meshes, uint32_t n, const int32_t *chunk_positions,
                        hc_mesh_info *out, void *stream) {
	if (!ctx || (n && (!meshes || !chunk_positions || !out)))
		return HC_ERR_INVALID_ARG;
	if (!n)
		return HC_OK;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	k_mesh_infos<<<(n + 255) / 256, 256, 0, stream ? (cudaStream_t)stream : ctx->stream>>>(meshes, n, chunk_positions,
	                                                                                        out);
	HC_CUDA(ctx, cudaGetLastError());
	return HC_OK;
}

hc_status hc_pool_create(hc_ctx *ctx, uint32_t capacity, hc_pool **out) {
	if (!ctx || !out || capacity == 0)
		return HC_ERR_INVALID_ARG;
	*out = nullptr;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	hc_pool *p = new hc_pool();
	p->ctx = ctx;
	p->capacity = capacity;
	cudaError_t e = cudaMalloc(&p->d_blocks, (size_t)capacity * 32768 * sizeof(uint16_t));
	if (e == cudaSuccess)
		e = cudaMalloc(&p->d_heights, (size_t)capacity * 1024);
	if (e == cudaSuccess)
		e = cudaMalloc(&p->d_planes, (size_t)capacity * kPlaneStride * sizeof(uint32_t));
	if (e != cudaSuccess) {
		hc_pool_destroy(p);
		return fail(ctx, e == cudaErrorMemoryAllocation ? HC_ERR_OUT_OF_MEMORY : HC_ERR_CUDA,
		            std::string("pool allocation: ") + cudaGetErrorString(e));
	}
	*out = p;
	return HC_OK;
}

void hc_pool_destroy(hc_pool *pool) {
	if (!pool)
		return;
	cudaSetDevice(pool->ctx->device);
	cudaFree(pool->d_blocks);
	cudaFree(pool->d_heights);
	cudaFree(pool->d_planes);
	delete pool;
}

uint32_t hc_pool_capacity(const hc_pool *pool) { return pool ? pool->capacity : 0; }

hc_status hc_pool_buffers(const hc_pool *pool, uint16_t **blocks, int8_t **heights) {
	if (!pool || !blocks || !heights)
		return HC_ERR_INVALID_ARG;
	*blocks = pool->d_blocks;
	*heights = pool->d_heights;
	return HC_OK;
}

hc_status hc_pool_upload(hc_pool *pool, uint32_t first, uint32_t count, const uint16_t *blocks, const int8_t *heights,
                         int src_on_device, void *stream) {
	if (!pool || !blocks || !heights)
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = pool->ctx;
	if ((uint64_t)first + count > pool->capacity)
		return fail(ctx, HC_ERR_INVALID_ARG, "upload beyond the pool capacity");
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	const cudaMemcpyKind kind = src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	HC_CUDA(ctx, cudaMemcpyAsync(pool->d_blocks + (size_t)first * 32768, blocks, (size_t)count * 32768 * sizeof(uint16_t),
	                             kind, st));
	HC_CUDA(ctx, cudaMemcpyAsync(pool->d_heights + (size_t)first * 1024, heights, (size_t)count * 1024, kind, st));
	return HC_OK;
}

hc_status hc_pool_download(hc_pool *pool, uint32_t first, uint32_t count, uint16_t *blocks, int8_t *heights,
                           int dst_on_device, void *stream) {
	if (!pool || (!blocks && !heights))
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = pool->ctx;
	if ((uint64_t)first + count > pool->capacity)
		return fail(ctx, HC_ERR_INVALID_ARG, "download beyond the pool capacity");
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	const cudaMemcpyKind kind = dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	if (blocks)
		HC_CUDA(ctx, cudaMemcpyAsync(blocks, pool->d_blocks + (size_t)first * 32768,
		                             (size_t)count * 32768 * sizeof(uint16_t), kind, st));
	if (heights)
		HC_CUDA(ctx, cudaMemcpyAsync(heights, pool->d_heights + (size_t)first * 1024, (size_t)count * 1024, kind, st));
	HC_CUDA(ctx, cudaStreamSynchronize(st));
	return HC_OK;
}

namespace {

// The knobs of persistent variant v (include/hc_gb300.h, HC_VARIANT_*).
int variant_cluster(int v) { return v == HC_VARIANT_CLUSTER2 ? 2 : (v == HC_VARIANT_CLUSTER4 ? 4 : 0); }
bool variant_light_pass(int v) { return v != HC_VARIANT_WINDOW && !variant_cluster(v); }
uint32_t variant_claim(int v) { return v == HC_VARIANT_CLAIM2 ? 2u : (v == HC_VARIANT_CLAIM4 ? 4u : 1u); }
// quad records past shared memory are dropped and the emission merges again in windows
bool variant_no_scratch(int v) { return v == HC_VARIANT_NO_SCRATCH; }

Arena plan_arena(const hc_batch_plan *p) {
	Arena A{reinterpret_cast<uint2 *>(p->arena.vertices),
	        p->arena.indices,
	        p->arena.meshes,
	        p->d_state,
	        reinterpret_cast<unsigned int *>(p->d_state + 1),
	        p->arena.quad_capacity,
	        p->arena.mesh_capacity,
	        p->arena.results,
	        p->d_spill};
	if (p->mode == HC_BATCH_PERSISTENT && variant_no_scratch(p->variant))
		A.spill = nullptr;
	return A;
}

cudaLaunchConfig_t cluster_config(dim3 grid, size_t smem, cudaStream_t st, cudaLaunchAttribute *attr, int csize) {
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = dim3(kThreads);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = st;
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = (unsigned)csize;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cfg;
}

// CTAs of a persistent grid of the cluster kernel: as many clusters as fit at once.
int cluster_grid_size(hc_ctx *ctx, int csize, int sms) {
	cudaLaunchAttribute attr[1];
	cudaLaunchConfig_t cfg = cluster_config(dim3(csize * ((sms + csize - 1) / csize)), ctx->smem_bytes, nullptr, attr, csize);
	int clusters = 0;
	if (cudaOccupancyMaxActiveClusters(&clusters, k_mesh_cluster, &cfg) != cudaSuccess || clusters < 1)
		clusters = std::max(1, sms / csize);
	return clusters * csize;
}

// Numbers the batch's distinct slots 0..n_slots-1 (their order in `slots`), rewrites the neighbour
// table in those numbers and derives every batch chunk's face neighbours from the 3x3x3 blocks of
// the table's rows (two slots are face neighbours when some row holds both, one step apart), then
// allocates the light pass's level planes and light bytes.
cudaError_t plan_light_tables(hc_batch_plan *p, const std::vector<int32_t> &table, const std::vector<int32_t> &slots) {
	const uint32_t m = (uint32_t)slots.size();
	std::vector<int32_t> local(p->pool->capacity, -1);
	for (uint32_t i = 0; i < m; ++i)
		local[slots[i]] = (int32_t)i;
	std::vector<int32_t> nbr_local(table.size(), 0), nb6((size_t)m * 6, -1);
	const int kOff[3] = {1, -1, 0}; // neighbour index digit -> offset (common/include/common/Position.hpp:146-152)
	const auto digit = [](int off) { return off == 1 ? 0 : (off == -1 ? 1 : 2); };
	for (size_t row = 0; row < table.size() / 27; ++row) {
		const int32_t *t = table.data() + row * 27;
		bool ok = true;
		for (int k = 0; k < 27; ++k) {
			ok &= t[k] >= 0 && (uint32_t)t[k] < p->pool->capacity;
			nbr_local[row * 27 + k] = ok ? local[t[k]] : 0;
		}
		if (!ok)
			continue; // the mesher reports the bad slot
		for (int k = 0; k < 27; ++k) {
			const int o[3] = {kOff[k / 9], kOff[(k / 3) % 3], kOff[k % 3]}; // x, y, z
			for (int f = 0; f < 6; ++f) {
				int q[3] = {o[0], o[1], o[2]};
				q[f >> 1] += (f & 1) ? 1 : -1;
				if (q[0] < -1 || q[0] > 1 || q[1] < -1 || q[1] > 1 || q[2] < -1 || q[2] > 1)
					continue;
				const int j = digit(q[0]) * 9 + digit(q[1]) * 3 + digit(q[2]);
				int32_t &dst = nb6[(size_t)local[t[k]] * 6 + f];
				if (dst < 0)
					dst = local[t[j]];
			}
		}
	}
	cudaError_t e = cudaMalloc(&p->d_nb6, nb6.size() * sizeof(int32_t));
	if (e == cudaSuccess)
		e = cudaMemcpy(p->d_nb6, nb6.data(), nb6.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMalloc(&p->d_nbr_local, nbr_local.size() * sizeof(int32_t));
	if (e == cudaSuccess)
		e = cudaMemcpy(p->d_nbr_local, nbr_local.data(), nbr_local.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMalloc(&p->d_levels, (size_t)m * kLevelSlotWords * sizeof(uint32_t));
	if (e == cudaSuccess)
		e = cudaMalloc(&p->d_edges, (size_t)m * kEdgeSlotWords * sizeof(uint32_t));
	if (e == cudaSuccess) // the uniform-plane flags, then the neighbour-light bits (LightPass::near)
		e = cudaMalloc(&p->d_lflags, (size_t)m * 4 * sizeof(uint32_t));
	return e;
}

// In a stream capture an external record becomes an event-record node of the graph, so every
// replay of the graph records the stage boundaries.
// Outside a capture it is a plain record (the external flag is only valid while capturing).
hc_status stage_mark(hc_batch_plan *p, int i, cudaStream_t st) {
	if (!p->stage_ev[i])
		return HC_OK;
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	HC_CUDA(p->ctx, cudaStreamIsCapturing(st, &cs));
	if (cs == cudaStreamCaptureStatusActive)
		HC_CUDA(p->ctx, cudaEventRecordWithFlags(p->stage_ev[i], st, cudaEventRecordExternal));
	else
		HC_CUDA(p->ctx, cudaEventRecord(p->stage_ev[i], st));
	return HC_OK;
}

hc_status enqueue_plan(hc_batch_plan *p, cudaStream_t st) {
	hc_ctx *ctx = p->ctx;
	hc_status s = stage_mark(p, 0, st);
	if (s != HC_OK)
		return s;
	HC_CUDA(ctx, cudaMemsetAsync(p->d_state, 0, 4 * sizeof(unsigned long long), st));
	if (p->n_slots) {
		const uint64_t rows = (uint64_t)p->n_slots * kPlaneWords;
		const int blocks = (int)std::min<uint64_t>((rows + 255) / 256, (uint64_t)p->grid * 8);
		k_planes_pool<<<blocks, 256, 0, st>>>(p->pool->d_blocks, p->pool->d_heights, p->d_slots, p->n_slots, tables(ctx),
		                                     p->pool->d_planes);
		HC_CUDA(ctx, cudaGetLastError());
	}
	if (p->d_blank && p->n_slots && !variant_cluster(p->variant)) {
		k_blank_items<<<(p->n + 7) / 8, 256, 0, st>>>(p->pool->d_planes, p->pool->capacity, p->nbr, p->n, p->d_blank);
		HC_CUDA(ctx, cudaGetLastError());
	}
	if ((s = stage_mark(p, 1, st)) != HC_OK)
		return s;
	const bool light_pass = variant_light_pass(p->variant) && p->d_levels;
	if (light_pass) {
		const LightPass L{p->d_slots,  p->d_nb6,   p->pool->d_planes, p->pool->d_blocks, p->d_levels,
		                  p->d_edges, p->d_lflags, p->d_lflags + 2 * (size_t)p->n_slots, p->n_slots};
		HC_CUDA(ctx, cudaMemsetAsync(L.near, 0, 2 * (size_t)p->n_slots * sizeof(uint32_t), st));
		for (int t = kLevels; t >= 1; --t) {
			k_light_level<<<(2 * p->n_slots + kLightWarps - 1) / kLightWarps, kLightThreads, 0, st>>>(L, tables(ctx), t);
			HC_CUDA(ctx, cudaGetLastError());
		}
	}
	if ((s = stage_mark(p, 2, st)) != HC_OK)
		return s;
	const Arena A = plan_arena(p);
	unsigned int *work = reinterpret_cast<unsigned int *>(p->d_state + 2);
	unsigned int *failed = reinterpret_cast<unsigned int *>(p->d_state + 3);
	if (p->mode == HC_BATCH_PERSISTENT && variant_cluster(p->variant)) {
		const int csize = variant_cluster(p->variant);
		cudaLaunchAttribute attr[1];
		cudaLaunchConfig_t cfg = cluster_config(dim3(p->cluster_grid[p->variant]), ctx->smem_bytes, st, attr, csize);
		HC_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_mesh_cluster, (const uint16_t *)p->pool->d_blocks,
		                                (const int8_t *)p->pool->d_heights, (const uint32_t *)p->pool->d_planes,
		                                p->pool->capacity, p->nbr, p->n, (const uint32_t *)nullptr, work, failed,
		                                tables(ctx), A, (const uint32_t *)nullptr, (const uint32_t *)nullptr,
		                                (const int32_t *)nullptr, csize));
	} else if (p->mode == HC_BATCH_PERSISTENT) {
		k_mesh_batch<<<p->grid, kThreads, ctx->smem_bytes, st>>>(
		    p->pool->d_blocks, p->pool->d_heights, p->pool->d_planes, p->pool->capacity, p->nbr, p->n, nullptr, work,
		    failed, tables(ctx), A, light_pass ? p->d_levels : nullptr, light_pass ? p->d_edges : nullptr,
		    light_pass ? p->d_nbr_local : nullptr, light_pass ? p->d_lflags : nullptr, p->d_blank,
		    variant_claim(p->variant));
		HC_CUDA(ctx, cudaGetLastError());
	} else {
		for (uint32_t i = 0; i < p->n; ++i) {
			k_mesh_item<<<1, kThreads, ctx->smem_bytes, st>>>(p->pool->d_blocks, p->pool->d_heights, p->pool->d_planes,
			                                                  p->pool->capacity, p->nbr, i, failed, tables(ctx), A);
		}
		HC_CUDA(ctx, cudaGetLastError());
	}
	return stage_mark(p, 3, st);
}

} // namespace

hc_status hc_batch_plan_create(hc_ctx *ctx, hc_pool *pool, const int32_t *neighbours, uint32_t n,
                               const hc_batch_arena *arena, int mode, int ctas_per_sm, hc_batch_plan **out) {
	if (!ctx || !pool || !neighbours || !arena || !out || n == 0 || !arena->vertices || !arena->indices ||
	    !arena->meshes || !arena->results)
		return HC_ERR_INVALID_ARG;
	if (mode != HC_BATCH_PERSISTENT && mode != HC_BATCH_PER_CHUNK && mode != HC_BATCH_AUTO &&
	    !(mode >= HC_BATCH_VARIANT(0) && mode < HC_BATCH_VARIANT(HC_VARIANT_COUNT)))
		return fail(ctx, HC_ERR_INVALID_ARG, "unknown batch mode");
	const bool autotune = mode == HC_BATCH_AUTO;
	// the persistent variants to build: the light pass, one pinned variant, or (autotuning) all of them
	int first = HC_VARIANT_LIGHT_PASS, last = autotune ? HC_VARIANT_COUNT - 1 : HC_VARIANT_LIGHT_PASS;
	if (mode >= HC_BATCH_VARIANT(0))
		first = last = mode - HC_BATCH_VARIANT(0);
	if (autotune || mode >= HC_BATCH_VARIANT(0))
		mode = HC_BATCH_PERSISTENT;
	if ((reinterpret_cast<uintptr_t>(arena->vertices) & 15u) || (reinterpret_cast<uintptr_t>(arena->indices) & 3u))
		return fail(ctx, HC_ERR_INVALID_ARG, "vertices must be 16-byte and indices 4-byte aligned");
	if (arena->quad_capacity > 0xffffffffull / 6)
		return fail(ctx, HC_ERR_INVALID_ARG, "quad capacity exceeds the 32-bit index offsets");
	*out = nullptr;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	hc_batch_plan *p = new hc_batch_plan();
	p->ctx = ctx;
	p->pool = pool;
	p->nbr = neighbours;
	p->n = n;
	p->arena = *arena;
	p->mode = mode;
	int sms = 0, per_sm = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mesh_batch, kThreads, ctx->smem_bytes);
	if (per_sm < 1)
		per_sm = 1;
	if (ctas_per_sm > 0 && ctas_per_sm < per_sm)
		per_sm = ctas_per_sm;
	p->grid = sms * per_sm;
	p->cluster_grid[HC_VARIANT_CLUSTER2] = cluster_grid_size(ctx, 2, sms);
	p->cluster_grid[HC_VARIANT_CLUSTER4] = cluster_grid_size(ctx, 4, sms);
	hc_status s = HC_OK;
	// distinct valid slots named by the neighbour table
	std::vector<int32_t> table((size_t)n * 27);
	cudaError_t e = cudaMemcpy(table.data(), neighbours, table.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
	if (e == cudaSuccess) {
		std::vector<uint8_t> used(pool->capacity, 0);
		std::vector<int32_t> slots;
		for (int32_t v : table)
			if (v >= 0 && (uint32_t)v < pool->capacity && !used[v])
				used[v] = 1, slots.push_back(v);
		p->n_slots = (uint32_t)slots.size();
		e = cudaMalloc(&p->d_slots, std::max<size_t>(1, slots.size()) * sizeof(int32_t));
		if (e == cudaSuccess && !slots.empty())
			e = cudaMemcpy(p->d_slots, slots.data(), slots.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
		if (e == cudaSuccess && mode == HC_BATCH_PERSISTENT && !slots.empty())
			e = plan_light_tables(p, table, slots);
	}
	if (e == cudaSuccess)
		e = cudaMalloc(&p->d_state, 4 * sizeof(unsigned long long));
	if (e == cudaSuccess)
		e = cudaMallocHost(&p->h_state, 4 * sizeof(unsigned long long));
	if (e == cudaSuccess) { // one record scratch per CTA of the largest grid the plan launches
		const int ctas = mode == HC_BATCH_PER_CHUNK
		                     ? 1
		                     : std::max(p->grid, std::max(p->cluster_grid[HC_VARIANT_CLUSTER2],
		                                                  p->cluster_grid[HC_VARIANT_CLUSTER4]));
		e = cudaMalloc(&p->d_spill, (size_t)ctas * kSpillRecs * sizeof(uint2));
	}
	if (e == cudaSuccess && mode == HC_BATCH_PERSISTENT) // the one-CTA persistent kernel skips blank chunks
		e = cudaMalloc(&p->d_blank, n);
	for (int i = 0; i < 4 && e == cudaSuccess; ++i)
		e = cudaEventCreate(&p->stage_ev[i]);
	if (e == cudaSuccess && mode == HC_BATCH_PERSISTENT) {
		e = cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking);
		float best_ms = 0.f;
		for (int v = first; v <= last && e == cudaSuccess && s == HC_OK; ++v) {
			p->variant = v;
			cudaGraph_t graph = nullptr;
			cudaGraphExec_t exec = nullptr;
			e = cudaStreamBeginCapture(p->capture_stream, cudaStreamCaptureModeThreadLocal);
			if (e == cudaSuccess) {
				s = enqueue_plan(p, p->capture_stream);
				cudaError_t e2 = cudaStreamEndCapture(p->capture_stream, &graph);
				if (s == HC_OK)
					e = e2;
			}
			if (e == cudaSuccess && s == HC_OK)
				e = cudaGraphInstantiate(&exec, graph, 0);
			float ms = 0.f;
			if (e == cudaSuccess && s == HC_OK && autotune) { // one warm run, then the mean of two
				cudaEvent_t e0 = nullptr, e1 = nullptr;
				e = cudaEventCreate(&e0);
				if (e == cudaSuccess)
					e = cudaEventCreate(&e1);
				if (e == cudaSuccess)
					e = cudaGraphLaunch(exec, p->capture_stream);
				if (e == cudaSuccess)
					e = cudaEventRecord(e0, p->capture_stream);
				for (int r = 0; r < 2 && e == cudaSuccess; ++r)
					e = cudaGraphLaunch(exec, p->capture_stream);
				if (e == cudaSuccess)
					e = cudaEventRecord(e1, p->capture_stream);
				if (e == cudaSuccess)
					e = cudaEventSynchronize(e1);
				if (e == cudaSuccess)
					e = cudaEventElapsedTime(&ms, e0, e1);
				ms *= 0.5f;
				p->variant_ms[v] = ms;
				if (e0)
					cudaEventDestroy(e0);
				if (e1)
					cudaEventDestroy(e1);
			}
			if (e == cudaSuccess && s == HC_OK && (!p->exec || ms < best_ms)) {
				if (p->exec)
					cudaGraphExecDestroy(p->exec), cudaGraphDestroy(p->graph);
				p->exec = exec, p->graph = graph, best_ms = ms;
				exec = nullptr, graph = nullptr;
			}
			if (exec)
				cudaGraphExecDestroy(exec);
			if (graph)
				cudaGraphDestroy(graph);
		}
		if (autotune && e == cudaSuccess && s == HC_OK) { // the variant whose graph was kept
			for (int v = first; v <= last; ++v)
				if (p->variant_ms[v] == best_ms)
					p->variant = v;
		}
	}
	if (e != cudaSuccess || s != HC_OK) {
		if (s == HC_OK)
			s = fail(ctx, e == cudaErrorMemoryAllocation ? HC_ERR_OUT_OF_MEMORY : HC_ERR_CUDA,
			         std::string("batch plan: ") + cudaGetErrorString(e));
		hc_batch_plan_destroy(p);
		return s;
	}
	*out = p;
	return HC_OK;
}

hc_status hc_batch_plan_stage_ms(hc_batch_plan *plan, float ms[3]) {
	if (!plan || !ms)
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = plan->ctx;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	HC_CUDA(ctx, cudaEventSynchronize(plan->stage_ev[3]));
	for (int i = 0; i < 3; ++i)
		HC_CUDA(ctx, cudaEventElapsedTime(&ms[i], plan->stage_ev[i], plan->stage_ev[i + 1]));
	return HC_OK;
}

hc_status hc_batch_plan_variant(const hc_batch_plan *plan, int *variant, float ms[HC_VARIANT_COUNT]) {
	if (!plan)
		return HC_ERR_INVALID_ARG;
	if (variant)
		*variant = plan->variant;
	if (ms)
		for (int v = 0; v < HC_VARIANT_COUNT; ++v)
			ms[v] = plan->variant_ms[v];
	return HC_OK;
}

void hc_batch_plan_destroy(hc_batch_plan *plan) {
	if (!plan)
		return;
	cudaSetDevice(plan->ctx->device);
	if (plan->exec)
		cudaGraphExecDestroy(plan->exec);
	if (plan->graph)
		cudaGraphDestroy(plan->graph);
	if (plan->capture_stream)
		cudaStreamDestroy(plan->capture_stream);
	for (cudaEvent_t ev : plan->stage_ev)
		if (ev)
			cudaEventDestroy(ev);
	cudaFree(plan->d_slots);
	cudaFree(plan->d_nb6);
	cudaFree(plan->d_nbr_local);
	cudaFree(plan->d_levels);
	cudaFree(plan->d_edges);
	cudaFree(plan->d_lflags);
	cudaFree(plan->d_state);
	cudaFree(plan->d_spill);
	cudaFree(plan->d_blank);
	cudaFreeHost(plan->h_state);
	delete plan;
}

hc_status hc_batch_plan_launch(hc_batch_plan *plan, void *stream) {
	if (!plan)
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = plan->ctx;
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	plan->last = st;
	if (plan->exec) {
		HC_CUDA(ctx, cudaGraphLaunch(plan->exec, st));
		return HC_OK;
	}
	return enqueue_plan(plan, st);
}

hc_status hc_batch_plan_result(hc_batch_plan *plan, uint64_t *quads, uint32_t *meshes, uint32_t *failed_chunks) {
	if (!plan)
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = plan->ctx;
	cudaStream_t st = plan->last ? plan->last : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	HC_CUDA(ctx, cudaMemcpyAsync(plan->h_state, plan->d_state, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
	HC_CUDA(ctx, cudaStreamSynchronize(st));
	if (quads)
		*quads = plan->h_state[0];
	if (meshes)
		*meshes = (uint32_t)(plan->h_state[1] & 0xffffffffu);
	if (failed_chunks)
		*failed_chunks = (uint32_t)(plan->h_state[3] & 0xffffffffu);
	return (plan->h_state[0] > plan->arena.quad_capacity || (plan->h_state[1] & 0xffffffffu) > plan->arena.mesh_capacity)
	           ? fail(ctx, HC_ERR_CAPACITY, "batch arena too small")
	           : HC_OK;
}

hc_status hc_batch_plan_download_async(hc_batch_plan *plan, uint64_t quads, uint32_t meshes, uint32_t *vertices,
                                       uint16_t *indices, hc_mesh_desc *mesh_descs, uint32_t *results, void *stream) {
	if (!plan)
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = plan->ctx;
	if (quads > plan->arena.quad_capacity || meshes > plan->arena.mesh_capacity)
		return fail(ctx, HC_ERR_INVALID_ARG, "download beyond the arena");
	cudaStream_t st = stream ? (cudaStream_t)stream : (plan->last ? plan->last : ctx->stream);
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	if (vertices && quads)
		HC_CUDA(ctx, cudaMemcpyAsync(vertices, plan->arena.vertices, quads * 4 * sizeof(uint2), cudaMemcpyDeviceToHost, st));
	if (indices && quads)
		HC_CUDA(ctx, cudaMemcpyAsync(indices, plan->arena.indices, quads * 6 * sizeof(uint16_t), cudaMemcpyDeviceToHost, st));
	if (mesh_descs && meshes)
		HC_CUDA(ctx, cudaMemcpyAsync(mesh_descs, plan->arena.meshes, (size_t)meshes * sizeof(hc_mesh_desc),
		                             cudaMemcpyDeviceToHost, st));
	if (results)
		HC_CUDA(ctx, cudaMemcpyAsync(results, plan->arena.results, (size_t)plan->n * 5 * sizeof(uint32_t),
		                             cudaMemcpyDeviceToHost, st));
	return HC_OK;
}

hc_status hc_batch_plan_download(hc_batch_plan *plan, uint64_t quads, uint32_t meshes, uint32_t *vertices,
                                 uint16_t *indices, hc_mesh_desc *mesh_descs, uint32_t *results) {
	const hc_status s = hc_batch_plan_download_async(plan, quads, meshes, vertices, indices, mesh_descs, results, nullptr);
	if (s != HC_OK)
		return s;
	HC_CUDA(plan->ctx, cudaStreamSynchronize(plan->last ? plan->last : plan->ctx->stream));
	return HC_OK;
}

} // extern "C"

// ------------------------------------------------------------------------------------------------
// Worlds: edits, height recomputation and remeshing of the chunks they touch.
// ------------------------------------------------------------------------------------------------
struct hc_world {
	hc_ctx *ctx = nullptr;
	hc_pool *pool = nullptr;
	hc_world_desc desc{};
	int cells = 0;
	uint32_t flood_words = 0, dirty_cap = 0;
	int32_t *d_slots = nullptr;
	uint32_t *d_flags = nullptr, *d_flood = nullptr, *d_stale = nullptr, *d_counts = nullptr;
	int32_t *d_dirty_list = nullptr, *d_flood_list = nullptr, *d_hchg_list = nullptr, *d_stale_list = nullptr;
	int32_t *d_list = nullptr, *d_nbr = nullptr;
	hc_edit *d_edits = nullptr;
	uint2 *d_sorted = nullptr;                  // one edit batch sorted by voxel, last edit of each voxel
	uint32_t *d_nsorted = nullptr;
	int32_t *d_stage = nullptr;                 // staged load/unload positions and slots
	unsigned long long *d_state = nullptr;      // arena cursors, work counter, failed count
	uint32_t *h_counts = nullptr;               // pinned
	unsigned long long *h_state = nullptr;      // pinned
	int32_t *h_stage = nullptr;                 // pinned, kStageChunks * 4
	int sms = 0;
	int cluster = 4;       // CTAs meshing one chunk (1: the one-CTA kernel)
	int cluster_grid = 0;  // CTAs of the cluster kernel's persistent grid
	uint2 *d_spill = nullptr; // quad records past the shared buffer, per CTA (at most one per SM)
};

namespace hc {
namespace detail {


constexpr uint32_t kStageChunks = 4096; // loads or unloads staged per launch
constexpr uint32_t kDirtySlack = 65536; // dirty-list room for cells unloaded and loaded again between collects

WorldDev world_dev(const hc_world *w) {
	WorldDev W;
	W.nx = w->desc.nx, W.ny = w->desc.ny, W.nz = w->desc.nz;
	W.cx0 = w->desc.cx0, W.cy0 = w->desc.cy0, W.cz0 = w->desc.cz0;
	W.slots = w->d_slots, W.flags = w->d_flags, W.flood = w->d_flood, W.stale = w->d_stale;
	W.blocks = w->pool->d_blocks, W.heights = w->pool->d_heights, W.pool_cap = w->pool->capacity;
	W.dirty_list = w->d_dirty_list, W.flood_list = w->d_flood_list, W.hchg_list = w->d_hchg_list;
	W.stale_list = w->d_stale_list, W.counts = w->d_counts, W.dirty_cap = w->dirty_cap;
	return W;
}

int list_grid(const hc_world *w) { return w->sms * 4; }

// Edits already on the device, then the height recompute they trigger.
hc_status world_enqueue_edits(hc_world *w, const hc_edit *d_edits, uint32_t n, cudaStream_t st) {
	hc_ctx *ctx = w->ctx;
	const WorldDev W = world_dev(w);
	for (uint32_t first = 0; first < n; first += kEditBatch) {
		k_sort_edits<<<1, kEditThreads, 0, st>>>(d_edits + first, std::min<uint32_t>(kEditBatch, n - first), W,
		                                         w->d_sorted, w->d_nsorted);
		HC_CUDA(ctx, cudaGetLastError());
		k_apply_sorted<<<std::min(w->sms * 2, (int)((n - first + 255) / 256)), 256, 0, st>>>(w->d_sorted, w->d_nsorted, W);
		HC_CUDA(ctx, cudaGetLastError());
	}
	return HC_OK;
}

hc_status world_enqueue_heights(hc_world *w, cudaStream_t st) {
	hc_ctx *ctx = w->ctx;
	const WorldDev W = world_dev(w);
	k_flood_columns<<<list_grid(w), 256, 0, st>>>(W, tables(ctx));
	HC_CUDA(ctx, cudaGetLastError());
	k_mark_heights<<<list_grid(w), 256, 0, st>>>(W);
	HC_CUDA(ctx, cudaGetLastError());
	return HC_OK;
}

// Everything of a remesh pass after the edits, reading every length on the device: the remesh list
// lands in w->d_list (length d_counts[kCountRemesh]).
hc_status world_enqueue_place(hc_world *w, const int32_t *d_pos, const int32_t *d_slots, uint32_t n, cudaStream_t st) {
	if (n) {
		k_place<<<(n + 255) / 256, 256, 0, st>>>(d_pos, d_slots, n, world_dev(w));
		HC_CUDA(w->ctx, cudaGetLastError());
	}
	return HC_OK;
}

hc_status world_enqueue_deltas(hc_world *w, const int32_t *d_slots, const uint32_t *d_boff, const uint32_t *d_soff,
                               const uint32_t *d_blocks, const uint16_t *d_suns, uint32_t n, cudaStream_t st) {
	if (n) {
		const Deltas D{d_slots, d_boff, d_soff, d_blocks, d_suns, n};
		k_apply_deltas<<<(n * 32 + 255) / 256, 256, 0, st>>>(D, w->pool->d_blocks, w->pool->d_heights);
		HC_CUDA(w->ctx, cudaGetLastError());
	}
	return HC_OK;
}

hc_status world_enqueue_evict(hc_world *w, const int32_t *d_pos, uint32_t n, cudaStream_t st) {
	if (n) {
		k_evict<<<(n + 255) / 256, 256, 0, st>>>(d_pos, n, world_dev(w));
		HC_CUDA(w->ctx, cudaGetLastError());
	}
	return HC_OK;
}

Arena world_arena(const hc_world *w, const hc_batch_arena *arena);

hc_status world_enqueue_remesh(hc_world *w, const hc_batch_arena *arena, cudaStream_t st) {
	hc_ctx *ctx = w->ctx;
	const WorldDev W = world_dev(w);
	const Arena A = world_arena(w, arena);
	k_planes_list<<<w->sms * 8, 256, 0, st>>>(W, tables(ctx), w->pool->d_planes);
	HC_CUDA(ctx, cudaGetLastError());
	k_collect<<<1, kEditThreads, kCollectSort * sizeof(uint32_t), st>>>(W, w->d_list, w->d_nbr);
	HC_CUDA(ctx, cudaGetLastError());
	HC_CUDA(ctx, cudaMemsetAsync(w->d_state, 0, 4 * sizeof(unsigned long long), st));
	unsigned int *work = reinterpret_cast<unsigned int *>(w->d_state + 2);
	unsigned int *failed = reinterpret_cast<unsigned int *>(w->d_state + 3);
	if (w->cluster > 1) {
		cudaLaunchAttribute attr[1];
		cudaLaunchConfig_t cfg = cluster_config(dim3(w->cluster_grid), ctx->smem_bytes, st, attr, w->cluster);
		HC_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_mesh_cluster, (const uint16_t *)w->pool->d_blocks,
		                                (const int8_t *)w->pool->d_heights, (const uint32_t *)w->pool->d_planes,
		                                w->pool->capacity, (const int32_t *)w->d_nbr, 0u,
		                                (const uint32_t *)(w->d_counts + kCountRemesh), work, failed, tables(ctx), A,
		                                (const uint32_t *)nullptr, (const uint32_t *)nullptr, (const int32_t *)nullptr,
		                                w->cluster));
	} else {
		k_mesh_batch<<<w->sms, kThreads, ctx->smem_bytes, st>>>(
		    w->pool->d_blocks, w->pool->d_heights, w->pool->d_planes, w->pool->capacity, w->d_nbr, 0u,
		    w->d_counts + kCountRemesh, work, failed, tables(ctx), A, nullptr, nullptr, nullptr, nullptr, nullptr, 1u);
	}
	HC_CUDA(ctx, cudaGetLastError());
	k_requeue<<<list_grid(w), 256, 0, st>>>(W, w->d_list, A.results);
	HC_CUDA(ctx, cudaGetLastError());
	return HC_OK;
}

hc_status world_enqueue_infos(hc_world *w, const hc_batch_arena *arena, int32_t *d_pos, hc_mesh_info *d_infos,
                              cudaStream_t st) {
	k_remesh_positions<<<(w->cells + 255) / 256, 256, 0, st>>>(world_dev(w), w->d_list, w->d_counts + kCountRemesh, d_pos);
	HC_CUDA(w->ctx, cudaGetLastError());
	k_mesh_infos_dev<<<std::max(1, std::min(w->sms * 4, (int)((arena->mesh_capacity + 255) / 256))), 256, 0, st>>>(
	    arena->meshes, reinterpret_cast<const unsigned int *>(w->d_state + 1), arena->mesh_capacity, d_pos, d_infos);
	HC_CUDA(w->ctx, cudaGetLastError());
	return HC_OK;
}

Arena world_arena(const hc_world *w, const hc_batch_arena *arena) {
	return Arena{reinterpret_cast<uint2 *>(arena->vertices),
	             arena->indices,
	             arena->meshes,
	             w->d_state,
	             reinterpret_cast<unsigned int *>(w->d_state + 1),
	             arena->quad_capacity,
	             arena->mesh_capacity,
	             arena->results,
	             w->d_spill};
}

hc_status check_arena(hc_ctx *ctx, const hc_batch_arena *arena, uint32_t cells) {
	if (!arena->vertices || !arena->indices || !arena->meshes || !arena->results)
		return fail(ctx, HC_ERR_INVALID_ARG, "arena buffers missing");
	if ((reinterpret_cast<uintptr_t>(arena->vertices) & 15u) || (reinterpret_cast<uintptr_t>(arena->indices) & 3u))
		return fail(ctx, HC_ERR_INVALID_ARG, "vertices must be 16-byte and indices 4-byte aligned");
	if (arena->quad_capacity > (1ull << 30))
		return fail(ctx, HC_ERR_INVALID_ARG, "arena quad capacity above 2^30");
	(void)cells;
	return HC_OK;
}

// Marks every resident slot's planes stale (after the pool was written outside the world's calls).
hc_status world_touch_all(hc_world *w, const int32_t *slots_host, cudaStream_t st) {
	hc_ctx *ctx = w->ctx;
	std::vector<uint8_t> seen(w->pool->capacity, 0);
	std::vector<int32_t> list;
	for (int i = 0; i < w->cells; ++i)
		if (slots_host[i] >= 0 && !seen[slots_host[i]])
			seen[slots_host[i]] = 1, list.push_back(slots_host[i]);
	const uint32_t n = (uint32_t)list.size();
	std::vector<uint32_t> flags(w->pool->capacity, 0);
	for (int32_t s : list)
		flags[s] = 1;
	HC_CUDA(ctx, cudaMemcpyAsync(w->d_stale, flags.data(), flags.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	if (n)
		HC_CUDA(ctx, cudaMemcpyAsync(w->d_stale_list, list.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
	HC_CUDA(ctx, cudaMemcpyAsync(w->d_counts + kCountStale, &n, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	HC_CUDA(ctx, cudaStreamSynchronize(st));
	return HC_OK;
}

const uint32_t *world_counts(const hc_world *w) { return w->d_counts; }
const int32_t *world_remesh_list(const hc_world *w) { return w->d_list; }
const unsigned long long *world_state(const hc_world *w) { return w->d_state; }
hc_pool *world_pool(const hc_world *w) { return w->pool; }
size_t pool_planes_bytes_per_slot() { return kPlaneStride * sizeof(uint32_t); }
hc_status ctx_fail(hc_ctx *ctx, hc_status s, const std::string &msg) { return fail(ctx, s, msg); }
int ctx_device(const hc_ctx *ctx) { return ctx->device; }

// Stages the stored edits of a group of loads (one device buffer for the call) and applies them;
// synchronous, as hc_world_load is.
hc_status load_deltas(hc_world *w, const hc_chunk_load *loads, uint32_t n, cudaStream_t st) {
	hc_ctx *ctx = w->ctx;
	std::vector<int32_t> slots;
	std::vector<uint32_t> boff(1, 0), soff(1, 0), blocks;
	std::vector<uint16_t> suns;
	for (uint32_t i = 0; i < n; ++i) {
		const hc_chunk_load &l = loads[i];
		if (!l.n_block_entries && !l.n_sunlight_entries)
			continue;
		slots.push_back(l.slot);
		blocks.insert(blocks.end(), l.block_entries, l.block_entries + l.n_block_entries);
		suns.insert(suns.end(), l.sunlight_entries, l.sunlight_entries + l.n_sunlight_entries);
		boff.push_back((uint32_t)blocks.size());
		soff.push_back((uint32_t)suns.size());
	}
	if (slots.empty())
		return HC_OK;
	const uint32_t m = (uint32_t)slots.size();
	const size_t bytes = m * 4 + 2 * (m + 1) * 4 + blocks.size() * 4 + suns.size() * 2 + 16;
	char *d = nullptr;
	HC_CUDA(ctx, cudaMalloc(&d, bytes));
	int32_t *d_slots = reinterpret_cast<int32_t *>(d);
	uint32_t *d_boff = reinterpret_cast<uint32_t *>(d_slots + m), *d_soff = d_boff + m + 1, *d_blocks = d_soff + m + 1;
	uint16_t *d_suns = reinterpret_cast<uint16_t *>(d_blocks + blocks.size());
	cudaError_t e = cudaMemcpyAsync(d_slots, slots.data(), m * 4, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d_boff, boff.data(), (m + 1) * 4, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d_soff, soff.data(), (m + 1) * 4, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess && !blocks.empty())
		e = cudaMemcpyAsync(d_blocks, blocks.data(), blocks.size() * 4, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess && !suns.empty())
		e = cudaMemcpyAsync(d_suns, suns.data(), suns.size() * 2, cudaMemcpyHostToDevice, st);
	hc_status s = e == cudaSuccess ? world_enqueue_deltas(w, d_slots, d_boff, d_soff, d_blocks, d_suns, m, st) : HC_OK;
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	cudaFree(d);
	if (e != cudaSuccess)
		return fail(ctx, HC_ERR_CUDA, std::string("load: stored edits: ") + cudaGetErrorString(e));
	return s;
}

} // namespace detail
} // namespace hc

using namespace hc::detail;

extern "C" {

hc_status hc_world_create(hc_ctx *ctx, hc_pool *pool, const hc_world_desc *desc, const int32_t *slots, hc_world **out) {
	if (!ctx || !pool || !desc || !slots || !out || desc->nx <= 0 || desc->ny <= 0 || desc->nz <= 0 || desc->ny > 32)
		return HC_ERR_INVALID_ARG;
	const long long cells = (long long)desc->nx * desc->ny * desc->nz;
	if (cells > (1ll << 21))
		return fail(ctx, HC_ERR_INVALID_ARG, "world grid larger than 2^21 chunks");
	for (long long i = 0; i < cells; ++i)
		if (slots[i] >= (int32_t)pool->capacity)
			return fail(ctx, HC_ERR_INVALID_ARG, "world slot beyond the pool capacity");
	*out = nullptr;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	hc_world *w = new hc_world();
	w->ctx = ctx, w->pool = pool, w->desc = *desc, w->cells = (int)cells;
	w->flood_words = (uint32_t)(desc->nx * desc->nz) * 1024u;
	w->dirty_cap = (uint32_t)cells + kDirtySlack;
	cudaDeviceGetAttribute(&w->sms, cudaDevAttrMultiProcessorCount, ctx->device);
	w->cluster_grid = cluster_grid_size(ctx, w->cluster, w->sms);
	cudaError_t e = cudaFuncSetAttribute(k_collect, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                     (int)(kCollectSort * sizeof(uint32_t)));
	const auto A = [&](void **p, size_t bytes) {
		if (e == cudaSuccess)
			e = cudaMalloc(p, bytes > 0 ? bytes : 1);
		if (e == cudaSuccess)
			e = cudaMemset(*p, 0, bytes > 0 ? bytes : 1);
	};
	A((void **)&w->d_slots, cells * sizeof(int32_t));
	A((void **)&w->d_spill, (size_t)w->sms * kSpillRecs * sizeof(uint2));
	A((void **)&w->d_flags, cells * sizeof(uint32_t));
	A((void **)&w->d_flood, (size_t)w->flood_words * sizeof(uint32_t));
	A((void **)&w->d_stale, (size_t)pool->capacity * sizeof(uint32_t));
	A((void **)&w->d_counts, kCountWords * sizeof(uint32_t));
	A((void **)&w->d_dirty_list, (size_t)w->dirty_cap * sizeof(int32_t));
	A((void **)&w->d_flood_list, (size_t)w->flood_words * sizeof(int32_t));
	A((void **)&w->d_hchg_list, cells * sizeof(int32_t));
	A((void **)&w->d_stale_list, (size_t)pool->capacity * sizeof(int32_t));
	A((void **)&w->d_list, cells * sizeof(int32_t));
	A((void **)&w->d_nbr, cells * 27 * sizeof(int32_t));
	A((void **)&w->d_edits, kEditBatch * sizeof(hc_edit));
	A((void **)&w->d_sorted, kEditBatch * sizeof(uint2));
	A((void **)&w->d_nsorted, sizeof(uint32_t));
	A((void **)&w->d_stage, kStageChunks * 4 * sizeof(int32_t));
	A((void **)&w->d_state, 4 * sizeof(unsigned long long));
	if (e == cudaSuccess)
		e = cudaMallocHost(&w->h_counts, kCountWords * sizeof(uint32_t));
	if (e == cudaSuccess)
		e = cudaMallocHost(&w->h_state, 4 * sizeof(unsigned long long));
	if (e == cudaSuccess)
		e = cudaMallocHost(&w->h_stage, kStageChunks * 4 * sizeof(int32_t));
	if (e == cudaSuccess)
		e = cudaMemcpy(w->d_slots, slots, cells * sizeof(int32_t), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		hc_world_destroy(w);
		return fail(ctx, e == cudaErrorMemoryAllocation ? HC_ERR_OUT_OF_MEMORY : HC_ERR_CUDA,
		            std::string("world: ") + cudaGetErrorString(e));
	}
	// every resident chunk's planes are built before the first remesh
	const hc_status s = world_touch_all(w, slots, ctx->stream);
	if (s != HC_OK) {
		hc_world_destroy(w);
		return s;
	}
	*out = w;
	return HC_OK;
}

void hc_world_destroy(hc_world *w) {
	if (!w)
		return;
	cudaSetDevice(w->ctx->device);
	for (void *p : {(void *)w->d_slots, (void *)w->d_flags, (void *)w->d_flood, (void *)w->d_stale, (void *)w->d_counts,
	                (void *)w->d_dirty_list, (void *)w->d_flood_list, (void *)w->d_hchg_list, (void *)w->d_stale_list,
	                (void *)w->d_list, (void *)w->d_nbr, (void *)w->d_edits, (void *)w->d_sorted, (void *)w->d_nsorted,
	                (void *)w->d_stage, (void *)w->d_state, (void *)w->d_spill})
		cudaFree(p);
	cudaFreeHost(w->h_counts);
	cudaFreeHost(w->h_state);
	cudaFreeHost(w->h_stage);
	delete w;
}

hc_status hc_world_apply_edits(hc_world *w, const hc_edit *edits, uint32_t n, int src_on_device, void *stream) {
	if (!w || (!edits && n))
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = w->ctx;
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	hc_status s;
	if (src_on_device) {
		if ((s = world_enqueue_edits(w, edits, n, st)) != HC_OK)
			return s;
	} else {
		for (uint32_t first = 0; first < n; first += kEditBatch) {
			const uint32_t nb = std::min<uint32_t>(kEditBatch, n - first);
			HC_CUDA(ctx, cudaMemcpyAsync(w->d_edits, edits + first, nb * sizeof(hc_edit), cudaMemcpyHostToDevice, st));
			if ((s = world_enqueue_edits(w, w->d_edits, nb, st)) != HC_OK)
				return s;
			HC_CUDA(ctx, cudaStreamSynchronize(st)); // d_edits is reused by the next batch
		}
	}
	return world_enqueue_heights(w, st);
}

hc_status hc_world_load(hc_world *w, const hc_chunk_load *loads, uint32_t n, void *stream) {
	if (!w || (!loads && n))
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = w->ctx;
	for (uint32_t i = 0; i < n; ++i)
		if (loads[i].slot < 0 || (uint32_t)loads[i].slot >= w->pool->capacity || !loads[i].blocks || !loads[i].heights)
			return fail(ctx, HC_ERR_INVALID_ARG, "load: slot beyond the pool or data missing");
	for (uint32_t i = 0; i < n; ++i)
		if ((loads[i].n_block_entries && !loads[i].block_entries) ||
		    (loads[i].n_sunlight_entries && !loads[i].sunlight_entries))
			return fail(ctx, HC_ERR_INVALID_ARG, "load: stored edits missing");
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	for (uint32_t first = 0; first < n; first += kStageChunks) {
		const uint32_t nb = std::min<uint32_t>(kStageChunks, n - first);
		for (uint32_t i = 0; i < nb; ++i) {
			const hc_chunk_load &l = loads[first + i];
			HC_CUDA(ctx, cudaMemcpyAsync(w->pool->d_blocks + (size_t)l.slot * 32768, l.blocks, 32768 * sizeof(uint16_t),
			                             cudaMemcpyHostToDevice, st));
			HC_CUDA(ctx, cudaMemcpyAsync(w->pool->d_heights + (size_t)l.slot * 1024, l.heights, 1024,
			                             cudaMemcpyHostToDevice, st));
			w->h_stage[3 * i] = l.cx, w->h_stage[3 * i + 1] = l.cy, w->h_stage[3 * i + 2] = l.cz;
			w->h_stage[3 * nb + i] = l.slot;
		}
		hc_status s = load_deltas(w, loads + first, nb, st); // after the chunk data, before the placing
		if (s != HC_OK)
			return s;
		HC_CUDA(ctx, cudaMemcpyAsync(w->d_stage, w->h_stage, 4 * nb * sizeof(int32_t), cudaMemcpyHostToDevice, st));
		s = world_enqueue_place(w, w->d_stage, w->d_stage + 3 * nb, nb, st);
		if (s != HC_OK)
			return s;
		HC_CUDA(ctx, cudaStreamSynchronize(st)); // the staging buffers are reused
	}
	return HC_OK;
}

hc_status hc_world_unload(hc_world *w, const int32_t *positions, uint32_t n, void *stream) {
	if (!w || (!positions && n))
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = w->ctx;
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	for (uint32_t first = 0; first < n; first += kStageChunks) {
		const uint32_t nb = std::min<uint32_t>(kStageChunks, n - first);
		std::memcpy(w->h_stage, positions + 3 * (size_t)first, 3 * nb * sizeof(int32_t));
		HC_CUDA(ctx, cudaMemcpyAsync(w->d_stage, w->h_stage, 3 * nb * sizeof(int32_t), cudaMemcpyHostToDevice, st));
		const hc_status s = world_enqueue_evict(w, w->d_stage, nb, st);
		if (s != HC_OK)
			return s;
		HC_CUDA(ctx, cudaStreamSynchronize(st));
	}
	return HC_OK;
}

hc_status hc_world_set_cluster(hc_world *w, int ctas_per_chunk) {
	if (!w || (ctas_per_chunk != 1 && ctas_per_chunk != 2 && ctas_per_chunk != 4 && ctas_per_chunk != 8))
		return HC_ERR_INVALID_ARG;
	w->cluster = ctas_per_chunk;
	w->cluster_grid = ctas_per_chunk > 1 ? cluster_grid_size(w->ctx, ctas_per_chunk, w->sms) : 0;
	return HC_OK;
}

hc_status hc_world_touch(hc_world *w, void *stream) {
	if (!w)
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = w->ctx;
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	std::vector<int32_t> slots(w->cells);
	HC_CUDA(ctx, cudaMemcpyAsync(slots.data(), w->d_slots, w->cells * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
	HC_CUDA(ctx, cudaStreamSynchronize(st));
	return world_touch_all(w, slots.data(), st);
}

hc_status hc_world_remesh(hc_world *w, const hc_batch_arena *arena, int32_t *cells, uint32_t cap, uint32_t *n_remeshed,
                          uint64_t *quads, uint32_t *meshes, void *stream) {
	if (!w || !arena || !n_remeshed || (!cells && cap))
		return HC_ERR_INVALID_ARG;
	hc_ctx *ctx = w->ctx;
	hc_status s = check_arena(ctx, arena, (uint32_t)w->cells);
	if (s != HC_OK)
		return s;
	if (cap < (uint32_t)w->cells)
		return fail(ctx, HC_ERR_INVALID_ARG, "cells must hold one entry per grid cell");
	cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
	HC_CUDA(ctx, cudaSetDevice(ctx->device));
	if ((s = world_enqueue_remesh(w, arena, st)) != HC_OK)
		return s;
	HC_CUDA(ctx, cudaMemcpyAsync(w->h_counts, w->d_counts, kCountWords * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	HC_CUDA(ctx, cudaMemcpyAsync(w->h_state, w->d_state, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
	HC_CUDA(ctx, cudaStreamSynchronize(st));
	const uint32_t n = w->h_counts[kCountRemesh];
	*n_remeshed = n;
	if (n) {
		HC_CUDA(ctx, cudaMemcpyAsync(cells, w->d_list, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
		HC_CUDA(ctx, cudaStreamSynchronize(st));
	}
	if (quads)
		*quads = std::min<unsigned long long>(w->h_state[0], arena->quad_capacity);
	if (meshes)
		*meshes = std::min<uint32_t>((uint32_t)(w->h_state[1] & 0xffffffffu), arena->mesh_capacity);
	if (w->h_state[3])
		return fail(ctx, HC_ERR_CAPACITY, std::to_string(w->h_state[3]) +
		                                      " chunks did not fit the arena; they stay marked for the next remesh");
	return HC_OK;
}

} // extern "C"

// ------------------------------------------------------------------------------------------------
// Meshing without device allocation.
//
// Some callers cannot call cudaMalloc: code that runs inside a host application's render or frame
// loop under a fixed device-memory budget, or a plugin whose host owns every device allocation. For
// them hc_mesh_batch_noalloc runs the batched kernel with its scratch (arena cursors, work counter,
// failed-chunk count and the five result words per chunk) and its block tables in file-scope
// device arrays below. Every GPU that loads this library holds them (about 390 KB) until exit.
// ------------------------------------------------------------------------------------------------
namespace {

constexpr uint32_t kNoAllocMaxChunks = HC_NOALLOC_MAX_CHUNKS;
constexpr uint32_t kNoAllocStateWords = 8; // quad cursor (u64), mesh cursor (u64), work counter, failed count

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocStateWords + 5 * kNoAllocMaxChunks];
static __device__ __align__(256) uint8_t g_noalloc_class_of[65536];
static __device__ __align__(256) DevClass g_noalloc_classes[256];

constexpr int kNoAllocMaxDevices = 64;
struct NoAllocDevice {
	bool ready;
	int sms;
	uint32_t *scratch;
	uint8_t *class_of;
	DevClass *classes;
};
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];
std::mutex g_noalloc_mutex;

// Host copies of the tables, in static storage (no heap).
hc_registry g_noalloc_registry;
uint8_t g_noalloc_class_of_host[65536];
DevClass g_noalloc_classes_host[256];
bool g_noalloc_tables_built = false;

bool noalloc_build_tables() {
	if (g_noalloc_tables_built)
		return true;
	hc_registry_build(&g_noalloc_registry);
	if (!assign_classes(g_noalloc_registry, g_noalloc_class_of_host, g_noalloc_classes_host))
		return false;
	g_noalloc_tables_built = true;
	return true;
}

// Writes a message into the caller's buffer (no heap use on any path of this entry point).
void noalloc_error(char *text, size_t size, const char *fmt, const char *arg = "", unsigned long long a = 0,
                   unsigned long long b = 0) {
	if (text && size)
		std::snprintf(text, size, fmt, arg, a, b);
}

// Once per device, with that device current: tables, kernel attribute, symbol addresses.
hc_status noalloc_setup(int dev, char *err, size_t err_size) {
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	NoAllocDevice &D = g_noalloc_dev[dev];
	if (D.ready)
		return HC_OK;
	if (!noalloc_build_tables()) {
		noalloc_error(err, err_size, "%smore than 256 distinct block classes");
		return HC_ERR_INVALID_ARG;
	}
	if (g_noalloc_registry.static_face_count > HC_MAX_STATIC_FACES / 4) {
		noalloc_error(err, err_size, "%stoo many static custom-mesh faces (%llu, at most %llu)", "",
		              (unsigned long long)g_noalloc_registry.static_face_count,
		              (unsigned long long)(HC_MAX_STATIC_FACES / 4));
		return HC_ERR_INVALID_ARG;
	}
	uint64_t tt = 0, tl = 0, tp = 0;
	for (int t = 0; t < HC_TEX_COUNT; ++t) {
		tt |= (uint64_t)hc_tex_is_transparent((uint16_t)t) << t;
		tl |= (uint64_t)hc_tex_is_liquid((uint16_t)t) << t;
		tp |= (uint64_t)hc_tex_use_transparent_pass((uint16_t)t) << t;
	}
	cudaError_t e = cudaFuncSetAttribute(k_mesh_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem));
	if (e == cudaSuccess)
		e = cudaMemcpyToSymbol(g_noalloc_class_of, g_noalloc_class_of_host, sizeof(g_noalloc_class_of_host));
	if (e == cudaSuccess)
		e = cudaMemcpyToSymbol(g_noalloc_classes, g_noalloc_classes_host, sizeof(g_noalloc_classes_host));
	if (e == cudaSuccess)
		e = cudaMemcpyToSymbol(c_tex_transparent, &tt, sizeof(tt));
	if (e == cudaSuccess)
		e = cudaMemcpyToSymbol(c_tex_liquid, &tl, sizeof(tl));
	if (e == cudaSuccess)
		e = cudaMemcpyToSymbol(c_tex_transpass, &tp, sizeof(tp));
	if (e == cudaSuccess)
		e = cudaMemcpyToSymbol(c_static_faces, g_noalloc_registry.static_faces,
		                       sizeof(hc_mesh_face) * g_noalloc_registry.static_face_count);
	// In host code the arrays' names are host-side stand-ins; the kernel gets their device addresses.
	if (e == cudaSuccess)
		e = cudaGetSymbolAddress((void **)&D.scratch, g_noalloc_scratch);
	if (e == cudaSuccess)
		e = cudaGetSymbolAddress((void **)&D.class_of, g_noalloc_class_of);
	if (e == cudaSuccess)
		e = cudaGetSymbolAddress((void **)&D.classes, g_noalloc_classes);
	if (e == cudaSuccess)
		e = cudaDeviceGetAttribute(&D.sms, cudaDevAttrMultiProcessorCount, dev);
	if (e != cudaSuccess) {
		noalloc_error(err, err_size, "no-alloc set-up: %s", cudaGetErrorString(e));
		return HC_ERR_CUDA;
	}
	D.ready = true;
	return HC_OK;
}

} // namespace

extern "C" hc_status hc_mesh_batch_noalloc(const uint16_t *pool_blocks, const int8_t *pool_heights, uint32_t pool_capacity,
                                           const int32_t *neighbours, uint32_t n, uint32_t *vertices, uint16_t *indices,
                                           hc_mesh_desc *meshes, uint64_t quad_capacity, uint32_t mesh_capacity,
                                           uint32_t *results_host, uint64_t *quads, uint32_t *mesh_count,
                                           uint32_t *failed_chunks, void *stream, char *error_text,
                                           size_t error_text_size) {
	noalloc_error(error_text, error_text_size, "%s");
	if (!pool_blocks || !pool_heights || !neighbours || !vertices || !indices || !meshes || pool_capacity == 0) {
		noalloc_error(error_text, error_text_size, "%snull buffer or empty pool");
		return HC_ERR_INVALID_ARG;
	}
	if (n == 0 || n > kNoAllocMaxChunks) {
		noalloc_error(error_text, error_text_size, "%sbatch of %llu chunks: the no-alloc path takes 1..%llu chunks per call", "",
		              (unsigned long long)n, (unsigned long long)kNoAllocMaxChunks);
		return HC_ERR_CAPACITY;
	}
	if ((reinterpret_cast<uintptr_t>(vertices) & 15u) || (reinterpret_cast<uintptr_t>(indices) & 3u)) {
		noalloc_error(error_text, error_text_size, "%svertices must be 16-byte and indices 4-byte aligned");
		return HC_ERR_INVALID_ARG;
	}
	if (quad_capacity > 0xffffffffull / 6) {
		noalloc_error(error_text, error_text_size, "%squad capacity exceeds the 32-bit index offsets");
		return HC_ERR_INVALID_ARG;
	}
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
		noalloc_error(error_text, error_text_size, "%sno current CUDA device");
		return HC_ERR_NO_DEVICE;
	}
	hc_status s = noalloc_setup(dev, error_text, error_text_size);
	if (s != HC_OK)
		return s;
	const NoAllocDevice &D = g_noalloc_dev[dev];
	cudaStream_t st = (cudaStream_t)stream;
	uint32_t *state = D.scratch;
	uint32_t *results = D.scratch + kNoAllocStateWords;
	// the array keeps the previous call's contents: the cursors and counters must start at zero
	e = cudaMemsetAsync(state, 0, kNoAllocStateWords * sizeof(uint32_t), st);
	if (e == cudaSuccess) {
		Arena A{reinterpret_cast<uint2 *>(vertices),
		        indices,
		        meshes,
		        reinterpret_cast<unsigned long long *>(state),
		        state + 2,
		        quad_capacity,
		        mesh_capacity,
		        results};
		k_mesh_batch<<<D.sms, kThreads, sizeof(Smem), st>>>(pool_blocks, pool_heights, nullptr, pool_capacity, neighbours,
		                                                     n, nullptr, state + 4, state + 5, DevTables{D.class_of, D.classes}, A,
		                                                     nullptr, nullptr, nullptr, nullptr, nullptr, 1u);
		e = cudaGetLastError();
	}
	uint32_t host_state[kNoAllocStateWords];
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(host_state, state, sizeof(host_state), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess && results_host)
		e = cudaMemcpyAsync(results_host, results, (size_t)n * 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) {
		noalloc_error(error_text, error_text_size, "no-alloc batch: %s", cudaGetErrorString(e));
		return HC_ERR_CUDA;
	}
	uint64_t q;
	std::memcpy(&q, host_state, sizeof(q));
	if (quads)
		*quads = q;
	if (mesh_count)
		*mesh_count = host_state[2];
	if (failed_chunks)
		*failed_chunks = host_state[5];
	if (q > quad_capacity || host_state[2] > mesh_capacity) {
		noalloc_error(error_text, error_text_size, "%soutput buffers too small; the required sizes are written back");
		return HC_ERR_CAPACITY;
	}
	return HC_OK;
}
