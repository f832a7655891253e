// Block edits, chunk loads and unloads on a resident world: apply, recompute sunlight heights,
// collect the chunks to remesh.
//
// The reference runs this as a chain of tasks per chunk: kSetBlock (client/src/ChunkSetBlockTask.cpp:
// 37-131) writes the blocks, marks the chunks to remesh with ChunkShouldRemesh
// (client/include/client/ChunkMeshTask.inl:9-15) and floods the edited columns; kFloodSunlight
// (client/src/ChunkFloodSunlightTask.cpp:33-66) recomputes their heights from the chunk above;
// kSetSunlight (client/src/ChunkSetSunlightTask.cpp:28-90) stores changed heights, marks the 27
// chunks around for remeshing and floods the same columns of the chunk below; kGenerate
// (client/src/ChunkGenerateTask.cpp:21-40) queues kMesh for the chunk it loaded, and kMesh waits
// until all 26 neighbours are loaded (client/src/ChunkMeshTask.cpp:14-39).
//
// Here each stage is a kernel over a device list that the stage before it appended to, with the
// list lengths in device memory, so a whole edit + remesh pass is enqueued without the host
// reading anything back:
//   edits / loads / unloads -> flood list, dirty list, stale-planes list
//   k_flood_columns         -> height-change list, stale-planes list
//   k_mark_heights          -> dirty list
//   k_collect               -> remesh list (grid order) + neighbour slot rows
//   k_planes_list           -> planes of every slot whose blocks or heights changed
//   k_mesh_batch, k_requeue -> chunks that did not fit the arena go back on the dirty list
// A consumer empties its list when its last block finishes (retire_list).
#pragma once
#include "hc_device.cuh"

namespace hc {

// Per grid cell state bits.
enum : uint32_t {
	kCellListed = 1u,  // on the dirty list (marked for remeshing)
	kCellWaiting = 2u, // marked, but a neighbour was missing at the last collect
	kCellHChg = 4u,    // on the height-change list
};

struct WorldDev {
	int nx, ny, nz, cx0, cy0, cz0;
	int32_t *slots;       // per grid cell, -1 when not resident
	uint32_t *flags;      // per grid cell, kCell* bits
	uint32_t *flood;      // per (cell column, x, z): bit iy set when layer iy was edited
	uint32_t *stale;      // per pool slot: on the stale-planes list
	uint16_t *blocks;     // pool
	int8_t *heights;      // pool
	uint32_t pool_cap;
	int32_t *dirty_list;  // grid cells, capacity dirty_cap
	int32_t *flood_list;  // flood words
	int32_t *hchg_list;   // grid cells
	int32_t *stale_list;  // pool slots
	uint32_t *counts;     // kCount* below
	uint32_t dirty_cap;
};

enum : int {
	kCountDirty = 0,   // appended to dirty_list (may exceed dirty_cap: then the collect scans the grid)
	kCountFlood = 1,
	kCountHChg = 2,
	kCountStale = 3,
	kCountRemesh = 4,  // chunks in the remesh list of the last collect
	kDoneFlood = 5,    // blocks of the list's consumer that finished (retire_list)
	kDoneHChg = 6,
	kDoneStale = 7,
	kCountWords = 8,
};

// Called by every block of a list's consumer kernel at its end: the last block to finish empties
// the list, after every block has read its length.
__device__ __forceinline__ void retire_list(uint32_t *counts, int count, int done) {
	__syncthreads();
	if (threadIdx.x == 0) {
		__threadfence();
		if (atomicAdd(counts + done, 1u) == gridDim.x - 1) {
			counts[count] = 0;
			counts[done] = 0;
			__threadfence();
		}
	}
}

constexpr int kEditBatch = 4096;
constexpr int kEditThreads = 1024;
constexpr int kCollectSort = 16384; // dirty lists up to this length are sorted in shared memory

__device__ __forceinline__ int floor_div32(int v) { return v >= 0 ? v / 32 : -((-v + 31) / 32); }
__device__ __forceinline__ int cell_of(const WorldDev &W, int ix, int iy, int iz) { return ix + W.nx * (iz + W.nz * iy); }
__device__ __forceinline__ bool in_grid(const WorldDev &W, int ix, int iy, int iz) {
	return ix >= 0 && iy >= 0 && iz >= 0 && ix < W.nx && iy < W.ny && iz < W.nz;
}
__device__ __forceinline__ void cell_xyz(const WorldDev &W, int cell, int &ix, int &iy, int &iz) {
	ix = cell % W.nx, iz = (cell / W.nx) % W.nz, iy = cell / (W.nx * W.nz);
}

// Marks a cell for remeshing; each cell is on the dirty list at most once while marked.
__device__ __forceinline__ void mark_dirty(const WorldDev &W, int cell) {
	if (!(atomicOr(W.flags + cell, kCellListed) & kCellListed)) {
		const uint32_t pos = atomicAdd(W.counts + kCountDirty, 1u);
		if (pos < W.dirty_cap)
			W.dirty_list[pos] = cell;
	}
}

// Marks a pool slot whose blocks or heights changed; its planes are rebuilt before the next mesh.
__device__ __forceinline__ void mark_stale(const WorldDev &W, int32_t slot) {
	if (!atomicOr(W.stale + slot, 1u))
		W.stale_list[atomicAdd(W.counts + kCountStale, 1u)] = slot;
}

// ChunkShouldRemesh: IsBorderLightInterfere at level 15 against [-1, 33)^3.
__device__ __forceinline__ bool should_remesh(int x, int y, int z) {
	const auto d = [](int v) { return v < -1 ? -1 - v : (v >= 33 ? v - 33 : 0); };
	return 15 > d(x) + d(y) + d(z);
}

// Sorts key[0, p) ascending (p a power of two) with all threads of the block.
template <typename K> __device__ void block_bitonic_sort(K *key, int p) {
	for (int size = 2; size <= p; size <<= 1)
		for (int stride = size >> 1; stride > 0; stride >>= 1) {
			for (int i = threadIdx.x; i < p; i += blockDim.x) {
				const int j = i ^ stride;
				if (j > i) {
					const K a = key[i], b = key[j];
					if ((a > b) == ((i & size) == 0)) {
						key[i] = b;
						key[j] = a;
					}
				}
			}
			__syncthreads();
		}
}

__device__ __forceinline__ int pow2_at_least(uint32_t n, int lo) {
	int p = lo;
	while ((uint32_t)p < n)
		p <<= 1;
	return p;
}

// Block-wide ordered compaction step: returns this thread's output position among the takers of
// this pass and advances *base by their number.
__device__ __forceinline__ uint32_t block_compact(bool take, uint32_t *s_warp, uint32_t &base) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t bal = __ballot_sync(0xffffffffu, take);
	if (lane == 0)
		s_warp[warp] = __popc(bal);
	__syncthreads();
	uint32_t before = 0, total = 0;
	for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
		before += w < warp ? s_warp[w] : 0;
		total += s_warp[w];
	}
	const uint32_t pos = base + before + __popc(bal & ((1u << lane) - 1u));
	__syncthreads();
	base += total;
	return pos;
}

// Sorts up to kEditBatch edits by (voxel, order) in shared memory and keeps the last edit of each
// voxel: out[0, *n_out) = (cell, voxel | block << 15). One CTA.
__global__ void __launch_bounds__(kEditThreads) k_sort_edits(const hc_edit *edits, uint32_t n, WorldDev W, uint2 *out,
                                                             uint32_t *n_out) {
	__shared__ unsigned long long key[kEditBatch];
	__shared__ uint32_t s_warp[kEditThreads / 32];
	const int tid = threadIdx.x;
	const int p = pow2_at_least(n, 32);
	for (int i = tid; i < p; i += kEditThreads) {
		unsigned long long k = ~0ull;
		if ((uint32_t)i < n) {
			const hc_edit e = edits[i];
			const int ix = floor_div32(e.x) - W.cx0, iy = floor_div32(e.y) - W.cy0, iz = floor_div32(e.z) - W.cz0;
			if (in_grid(W, ix, iy, iz)) {
				const int cell = cell_of(W, ix, iy, iz);
				if (W.slots[cell] >= 0) {
					const uint32_t lidx = (uint32_t)((e.x & 31) + ((e.y & 31) * 32 + (e.z & 31)) * 32);
					k = ((unsigned long long)cell << 27) | ((unsigned long long)lidx << 12) | (unsigned long long)i;
				}
			}
		}
		key[i] = k;
	}
	__syncthreads();
	block_bitonic_sort(key, p);
	uint32_t base = 0;
	for (int i0 = 0; i0 < p; i0 += kEditThreads) {
		const int i = i0 + tid;
		const unsigned long long k = i < p ? key[i] : ~0ull;
		// a later edit of the same voxel wins
		const bool take = k != ~0ull && !(i + 1 < p && (key[i + 1] >> 12) == (k >> 12));
		const uint32_t pos = block_compact(take, s_warp, base);
		if (take)
			out[pos] = make_uint2((uint32_t)(k >> 27), (uint32_t)((k >> 12) & 32767u) | ((edits[k & 4095u].block & 0xffffu) << 15));
	}
	if (tid == 0)
		*n_out = base;
}

// Writes each sorted edit's voxel, marking remeshes and floods as ChunkSetBlockTask.cpp:83-107
// does for a block that changed. Grid-stride over the sorted edits.
__global__ void k_apply_sorted(const uint2 *sorted, const uint32_t *n_sorted, WorldDev W) {
	const uint32_t n = *n_sorted;
	for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
		const uint2 v = sorted[e];
		const int cell = (int)v.x, lidx = (int)(v.y & 32767u);
		const uint16_t nb = (uint16_t)(v.y >> 15);
		const int32_t slot = W.slots[cell];
		uint16_t *dst = W.blocks + (size_t)slot * 32768 + lidx;
		if (*dst == nb)
			continue;
		*dst = nb;
		mark_stale(W, slot);
		int ix, iy, iz;
		cell_xyz(W, cell, ix, iy, iz);
		const int lx = lidx & 31, lz = (lidx >> 5) & 31, ly = lidx >> 10;
		for (int d = 0; d < 27; ++d) {
			const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
			if (in_grid(W, ix + dx, iy + dy, iz + dz) && should_remesh(lx - 32 * dx, ly - 32 * dy, lz - 32 * dz))
				mark_dirty(W, cell_of(W, ix + dx, iy + dy, iz + dz));
		}
		const uint32_t word = (uint32_t)(ix + W.nx * iz) * 1024u + (uint32_t)(lx + 32 * lz);
		if (!atomicOr(W.flood + word, 1u << iy))
			W.flood_list[atomicAdd(W.counts + kCountFlood, 1u)] = (int32_t)word;
	}
}

// Puts n chunks into the grid: chunk (pos[3i], pos[3i+1], pos[3i+2]) now lives in pool slot
// slot[i] (its blocks and heights already there). The chunk is marked for remeshing (kGenerate
// queues kMesh for itself), and each neighbour that was waiting for a missing neighbour is marked
// again. Positions outside the grid are skipped.
__global__ void k_place(const int32_t *pos, const int32_t *slot, uint32_t n, WorldDev W) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const int ix = pos[3 * i] - W.cx0, iy = pos[3 * i + 1] - W.cy0, iz = pos[3 * i + 2] - W.cz0;
	const int32_t s = slot[i];
	if (!in_grid(W, ix, iy, iz) || s < 0 || (uint32_t)s >= W.pool_cap)
		return;
	const int cell = cell_of(W, ix, iy, iz);
	W.slots[cell] = s;
	mark_stale(W, s);
	mark_dirty(W, cell);
	for (int d = 0; d < 27; ++d) {
		const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
		if (d == 13 || !in_grid(W, ix + dx, iy + dy, iz + dz))
			continue;
		const int nc = cell_of(W, ix + dx, iy + dy, iz + dz);
		if (atomicAnd(W.flags + nc, ~kCellWaiting) & kCellWaiting)
			mark_dirty(W, nc);
	}
}

// Stored edits of loaded chunks (common/include/common/Data.hpp:36-86): chunk k of the batch lives
// in slot[k]; its block entries are blocks[boff[k], boff[k + 1]) and its sunlight entries
// suns[soff[k], soff[k + 1]).
struct Deltas {
	const int32_t *slot;
	const uint32_t *boff, *soff;
	const uint32_t *blocks; // cell index << 16 | raw block
	const uint16_t *suns;   // column index << 6 | height
	uint32_t n;
};

// One warp per loaded chunk applies its entries in order, as ChunkTaskRunner<kGenerate>::Run
// calls SetBlock / SetSunlightHeight for each (client/src/ChunkGenerateTask.cpp:33-36): within
// each group of 32 the last entry of a cell wins, and groups go in order.
__global__ void k_apply_deltas(Deltas D, uint16_t *pool_blocks, int8_t *pool_heights) {
	const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (w >= D.n)
		return;
	const size_t slot = (size_t)D.slot[w];
	for (uint32_t i0 = D.boff[w]; i0 < D.boff[w + 1]; i0 += 32) {
		const uint32_t i = i0 + lane;
		const bool valid = i < D.boff[w + 1] && (D.blocks[i] >> 16) < 32768u;
		const uint32_t e = valid ? D.blocks[i] : 0u;
		const uint32_t peers = __match_any_sync(0xffffffffu, valid ? (e >> 16) : 0x10000u + lane);
		if (valid && lane == 31 - __clz(peers))
			pool_blocks[slot * 32768 + (e >> 16)] = (uint16_t)(e & 0xffffu);
		__syncwarp();
	}
	for (uint32_t i0 = D.soff[w]; i0 < D.soff[w + 1]; i0 += 32) {
		const uint32_t i = i0 + lane;
		const bool valid = i < D.soff[w + 1];
		const uint32_t e = valid ? D.suns[i] : 0u;
		const uint32_t peers = __match_any_sync(0xffffffffu, valid ? (e >> 6) : 0x10000u + lane);
		if (valid && lane == 31 - __clz(peers))
			pool_heights[slot * 1024 + (e >> 6)] = (int8_t)(e & 63u);
		__syncwarp();
	}
}

// Takes n chunks out of the grid (ChunkTaskData<kMesh>::OnUnload drops a queued remesh too).
__global__ void k_evict(const int32_t *pos, uint32_t n, WorldDev W) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const int ix = pos[3 * i] - W.cx0, iy = pos[3 * i + 1] - W.cy0, iz = pos[3 * i + 2] - W.cz0;
	if (!in_grid(W, ix, iy, iz))
		return;
	const int cell = cell_of(W, ix, iy, iz);
	W.slots[cell] = -1;
	atomicAnd(W.flags + cell, ~(kCellListed | kCellWaiting));
}

// One listed column (cell column, x, z) per thread, top to bottom: a layer is recomputed when it
// was edited or when the layer above changed (the kSetSunlight -> kFloodSunlight cascade); a
// changed height goes on the height-change list.
__global__ void k_flood_columns(WorldDev W, const DevTables T) {
	const uint32_t n = *(volatile uint32_t *)(W.counts + kCountFlood);
	for (uint32_t li = blockIdx.x * blockDim.x + threadIdx.x; li < n; li += gridDim.x * blockDim.x) {
		const uint32_t c = (uint32_t)W.flood_list[li];
		const uint32_t bits = W.flood[c];
		W.flood[c] = 0;
		if (!bits)
			continue;
		const int colxz = (int)(c >> 10), ix = colxz % W.nx, iz = colxz / W.nx;
		const int x = (int)(c & 31u), z = (int)((c >> 5) & 31u);
		bool cascade = false;
		for (int iy = 31 - __clz(bits); iy >= 0; --iy) {
			if (!cascade && !((bits >> iy) & 1u))
				continue;
			const int cell = cell_of(W, ix, iy, iz);
			const int32_t slot = W.slots[cell];
			if (slot < 0)
				break;
			const int32_t up = iy + 1 < W.ny ? W.slots[cell_of(W, ix, iy + 1, iz)] : -1;
			int8_t nh;
			if (up >= 0 && W.heights[(size_t)up * 1024 + x + 32 * z] > 0) {
				nh = 32;
			} else { // ChunkFloodSunlightTask.cpp:47-51
				const uint16_t *b = W.blocks + (size_t)slot * 32768 + x + 32 * z;
				int y = 31;
				while (y >= 0 && (T.classes[T.class_of[b[y * 1024]]].flags & kFVertical))
					--y;
				nh = (int8_t)(y + 1);
			}
			int8_t *h = W.heights + (size_t)slot * 1024 + x + 32 * z;
			cascade = *h != nh;
			if (cascade) {
				*h = nh;
				mark_stale(W, slot);
				if (!(atomicOr(W.flags + cell, kCellHChg) & kCellHChg))
					W.hchg_list[atomicAdd(W.counts + kCountHChg, 1u)] = cell;
			}
		}
	}
	retire_list(W.counts, kCountFlood, kDoneFlood);
}

// A chunk whose heights changed is remeshed with the 26 around it (ChunkSetSunlightTask.cpp:63-83).
__global__ void k_mark_heights(WorldDev W) {
	const uint32_t n = *(volatile uint32_t *)(W.counts + kCountHChg);
	for (uint32_t li = blockIdx.x * blockDim.x + threadIdx.x; li < n; li += gridDim.x * blockDim.x) {
		const int cell = W.hchg_list[li];
		atomicAnd(W.flags + cell, ~kCellHChg);
		int ix, iy, iz;
		cell_xyz(W, cell, ix, iy, iz);
		for (int d = 0; d < 27; ++d) {
			const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
			if (in_grid(W, ix + dx, iy + dy, iz + dz))
				mark_dirty(W, cell_of(W, ix + dx, iy + dy, iz + dz));
		}
	}
	retire_list(W.counts, kCountHChg, kDoneHChg);
}

// Decides one listed cell at collect time: true when it is resident and its 26 neighbours are
// (then it is remeshed now); a resident cell with a missing neighbour waits for a load next to it.
__device__ __forceinline__ bool collect_cell(const WorldDev &W, int cell) {
	if (W.slots[cell] < 0) {
		atomicAnd(W.flags + cell, ~(kCellListed | kCellWaiting));
		return false;
	}
	int ix, iy, iz;
	cell_xyz(W, cell, ix, iy, iz);
	bool all = ix > 0 && iy > 0 && iz > 0 && ix < W.nx - 1 && iy < W.ny - 1 && iz < W.nz - 1;
	if (all) {
		int32_t s[27]; // all loads in flight at once
#pragma unroll
		for (int d = 0; d < 27; ++d)
			s[d] = W.slots[cell_of(W, ix + d % 3 - 1, iy + (d / 3) % 3 - 1, iz + d / 9 - 1)];
#pragma unroll
		for (int d = 0; d < 27; ++d)
			all &= s[d] >= 0;
	}
	if (all)
		atomicAnd(W.flags + cell, ~(kCellListed | kCellWaiting));
	else
		atomicOr(W.flags + cell, kCellWaiting), atomicAnd(W.flags + cell, ~kCellListed);
	return all;
}

// Writes the remesh list entry pos: the cell and its 27 neighbour slots in the reference's
// neighbour order (common/include/common/Position.hpp:146-152), centre last.
__device__ __forceinline__ void write_remesh(const WorldDev &W, int cell, uint32_t pos, int32_t *list, int32_t *nbr) {
	list[pos] = cell;
	int ix, iy, iz;
	cell_xyz(W, cell, ix, iy, iz);
	const int kRev[3] = {1, -1, 0};
#pragma unroll
	for (int i = 0; i < 27; ++i) {
		const int dz = kRev[i % 3], dy = kRev[(i / 3) % 3], dx = kRev[i / 9];
		nbr[(size_t)pos * 27 + i] = W.slots[cell_of(W, ix + dx, iy + dy, iz + dz)];
	}
}

// Builds the remesh list, in grid order, from the dirty list (sorted in shared memory) or, when
// the list overflowed or is longer than kCollectSort, from a scan of every cell's flags. Retires
// the dirty and height-change lists. One CTA of kEditThreads threads, kCollectSort * 4 bytes of
// dynamic shared memory.
__global__ void __launch_bounds__(kEditThreads) k_collect(WorldDev W, int32_t *list, int32_t *nbr) {
	extern __shared__ uint32_t s_key[];
	__shared__ uint32_t s_warp[kEditThreads / 32];
	const int tid = threadIdx.x;
	const uint32_t nd = W.counts[kCountDirty];
	uint32_t base = 0;
	if (nd <= W.dirty_cap && nd <= (uint32_t)kCollectSort) {
		const int p = pow2_at_least(nd, 32);
		for (int i = tid; i < p; i += kEditThreads)
			s_key[i] = (uint32_t)i < nd ? (uint32_t)W.dirty_list[i] : 0xffffffffu;
		__syncthreads();
		block_bitonic_sort(s_key, p);
		for (int i0 = 0; i0 < p; i0 += kEditThreads) {
			const int i = i0 + tid;
			const uint32_t k = i < p ? s_key[i] : 0xffffffffu;
			const bool first = k != 0xffffffffu && (i == 0 || s_key[i - 1] != k);
			const bool take = first && collect_cell(W, (int)k);
			const uint32_t pos = block_compact(take, s_warp, base);
			if (take)
				write_remesh(W, (int)k, pos, list, nbr);
		}
	} else {
		const int cells = W.nx * W.ny * W.nz;
		for (int c0 = 0; c0 < cells; c0 += kEditThreads) {
			const int cell = c0 + tid;
			const bool take = cell < cells && (W.flags[cell] & kCellListed) && collect_cell(W, cell);
			const uint32_t pos = block_compact(take, s_warp, base);
			if (take)
				write_remesh(W, cell, pos, list, nbr);
		}
	}
	if (tid == 0) {
		W.counts[kCountRemesh] = base;
		W.counts[kCountDirty] = 0;
	}
}

// Planes of the slots on the stale list (grid-stride over slot x row); clears their marks.
__global__ void __launch_bounds__(256) k_planes_list(WorldDev W, DevTables T, uint32_t *planes) {
	__shared__ DevClass cls[256];
	for (int i = threadIdx.x; i < 256; i += blockDim.x)
		cls[i] = T.classes[i];
	__syncthreads();
	const uint64_t total = (uint64_t)*(volatile uint32_t *)(W.counts + kCountStale) * kPlaneWords;
	for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x) {
		const uint32_t i = (uint32_t)(g / kPlaneWords), r = (uint32_t)(g % kPlaneWords);
		const size_t slot = (size_t)W.stale_list[i];
		planes_row(W.blocks + slot * 32768, W.heights + slot * 1024, cls, T.class_of, (int)r, planes + slot * kPlaneStride);
		if (r == 0)
			W.stale[slot] = 0;
	}
	retire_list(W.counts, kCountStale, kDoneStale);
}

// After the batch: chunks that did not fit the arena go back on the dirty list.
__global__ void k_requeue(WorldDev W, const int32_t *list, const uint32_t *results) {
	const uint32_t n = W.counts[kCountRemesh];
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		if (results[5 * (size_t)i + 4] != 0)
			mark_dirty(W, list[i]);
}

} // namespace hc
