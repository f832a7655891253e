// Block edits on a resident world: apply, recompute sunlight heights, collect chunks to remesh.
//
// The reference runs this as a chain of tasks per chunk: kSetBlock (client/src/ChunkSetBlockTask.cpp:
// 37-131) writes the blocks, marks the chunks to remesh with ChunkShouldRemesh
// (client/include/client/ChunkMeshTask.inl:9-15) and floods the edited columns; kFloodSunlight
// (client/src/ChunkFloodSunlightTask.cpp:33-66) recomputes their heights from the chunk above;
// kSetSunlight (client/src/ChunkSetSunlightTask.cpp:28-90) stores changed heights, marks the 27
// chunks around for remeshing and floods the same columns of the chunk below. Here each stage is a
// kernel over the whole edit batch.
#pragma once
#include "hc_device.cuh"

namespace hc {

struct WorldDev {
	int nx, ny, nz, cx0, cy0, cz0;
	const int32_t *slots; // per grid cell, -1 when not resident
	uint8_t *dirty;       // per grid cell: to remesh
	uint8_t *hchg;        // per grid cell: a height changed in this pass
	uint32_t *flood;      // per (cell column, x, z): bit iy set when layer iy was edited
	uint16_t *blocks;     // pool
	int8_t *heights;      // pool
};

constexpr int kEditBatch = 4096;
constexpr int kEditThreads = 1024;

__device__ __forceinline__ int floor_div32(int v) { return v >= 0 ? v / 32 : -((-v + 31) / 32); }
__device__ __forceinline__ int cell_of(const WorldDev &W, int ix, int iy, int iz) { return ix + W.nx * (iz + W.nz * iy); }
__device__ __forceinline__ bool in_grid(const WorldDev &W, int ix, int iy, int iz) {
	return ix >= 0 && iy >= 0 && iz >= 0 && ix < W.nx && iy < W.ny && iz < W.nz;
}

// ChunkShouldRemesh: IsBorderLightInterfere at level 15 against [-1, 33)^3.
__device__ __forceinline__ bool should_remesh(int x, int y, int z) {
	const auto d = [](int v) { return v < -1 ? -1 - v : (v >= 33 ? v - 33 : 0); };
	return 15 > d(x) + d(y) + d(z);
}

// Applies up to kEditBatch edits: sorts them by (voxel, order) in shared memory so the last edit of
// a voxel wins, then writes each distinct voxel once, marking remeshes and floods as
// ChunkSetBlockTask.cpp:83-107 does for a block that changed.
__global__ void __launch_bounds__(kEditThreads) k_apply_edits(const hc_edit *edits, uint32_t n, WorldDev W) {
	__shared__ unsigned long long key[kEditBatch];
	const int tid = threadIdx.x;
	for (int i = tid; i < kEditBatch; i += kEditThreads) {
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
	for (int size = 2; size <= kEditBatch; size <<= 1) // bitonic sort, ascending
		for (int stride = size >> 1; stride > 0; stride >>= 1) {
			for (int i = tid; i < kEditBatch; i += kEditThreads) {
				const int j = i ^ stride;
				if (j > i) {
					const unsigned long long a = key[i], b = key[j];
					const bool up = (i & size) == 0;
					if ((a > b) == up) {
						key[i] = b;
						key[j] = a;
					}
				}
			}
			__syncthreads();
		}
	for (int i = tid; i < kEditBatch; i += kEditThreads) {
		const unsigned long long k = key[i];
		if (k == ~0ull)
			continue;
		if (i + 1 < kEditBatch && (key[i + 1] >> 12) == (k >> 12))
			continue; // a later edit of the same voxel wins
		const int cell = (int)(k >> 27), lidx = (int)((k >> 12) & 32767u), order = (int)(k & 4095u);
		const uint16_t nb = (uint16_t)(edits[order].block & 0xffffu);
		uint16_t *dst = W.blocks + (size_t)W.slots[cell] * 32768 + lidx;
		if (*dst == nb)
			continue;
		*dst = nb;
		const int ix = cell % W.nx, iz = (cell / W.nx) % W.nz, iy = cell / (W.nx * W.nz);
		const int lx = lidx & 31, lz = (lidx >> 5) & 31, ly = lidx >> 10;
		for (int d = 0; d < 27; ++d) {
			const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
			if (in_grid(W, ix + dx, iy + dy, iz + dz) && should_remesh(lx - 32 * dx, ly - 32 * dy, lz - 32 * dz))
				W.dirty[cell_of(W, ix + dx, iy + dy, iz + dz)] = 1;
		}
		atomicOr(W.flood + ((size_t)(ix + W.nx * iz) * 1024 + lx + 32 * lz), 1u << iy);
	}
}

// One column (cell column, x, z) per thread, top to bottom: a layer is recomputed when it was
// edited or when the layer above changed (the kSetSunlight -> kFloodSunlight cascade); a changed
// height marks its chunk.
__global__ void k_flood_columns(WorldDev W, const DevTables T) {
	const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= (uint32_t)(W.nx * W.nz) * 1024u)
		return;
	const uint32_t bits = W.flood[c];
	if (!bits)
		return;
	W.flood[c] = 0;
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
			W.hchg[cell] = 1;
		}
	}
}

// A chunk whose heights changed is remeshed with the 26 around it (ChunkSetSunlightTask.cpp:63-83).
__global__ void k_mark_heights(WorldDev W) {
	const int cell = blockIdx.x * blockDim.x + threadIdx.x;
	if (cell >= W.nx * W.ny * W.nz || !W.hchg[cell])
		return;
	W.hchg[cell] = 0;
	const int ix = cell % W.nx, iz = (cell / W.nx) % W.nz, iy = cell / (W.nx * W.nz);
	for (int d = 0; d < 27; ++d) {
		const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
		if (in_grid(W, ix + dx, iy + dy, iz + dz))
			W.dirty[cell_of(W, ix + dx, iy + dy, iz + dz)] = 1;
	}
}

// Lists, in grid order, the marked chunks whose 26 neighbours are resident, writes their neighbour
// slot rows (neighbour order, centre last), clears their marks and lists the distinct slots they
// read. count[0] = chunks, count[1] = slots. One CTA.
__global__ void __launch_bounds__(kEditThreads) k_collect(WorldDev W, int32_t *list, int32_t *nbr, uint8_t *slot_mark,
                                                          uint32_t pool_cap, int32_t *slot_list, uint32_t *count) {
	__shared__ uint32_t s_base, s_warp[kEditThreads / 32];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int cells = W.nx * W.ny * W.nz;
	if (tid == 0)
		s_base = 0;
	__syncthreads();
	for (int c0 = 0; c0 < cells; c0 += kEditThreads) {
		const int cell = c0 + tid;
		bool take = false;
		if (cell < cells && W.dirty[cell] && W.slots[cell] >= 0) {
			const int ix = cell % W.nx, iz = (cell / W.nx) % W.nz, iy = cell / (W.nx * W.nz);
			take = true;
			for (int d = 0; d < 27 && take; ++d) {
				const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
				take = in_grid(W, ix + dx, iy + dy, iz + dz) && W.slots[cell_of(W, ix + dx, iy + dy, iz + dz)] >= 0;
			}
		}
		const uint32_t bal = __ballot_sync(0xffffffffu, take);
		if (lane == 0)
			s_warp[warp] = __popc(bal);
		__syncthreads();
		uint32_t before = 0, total = 0;
		for (int w = 0; w < kEditThreads / 32; ++w) {
			before += w < warp ? s_warp[w] : 0;
			total += s_warp[w];
		}
		if (take) {
			const uint32_t pos = s_base + before + __popc(bal & ((1u << lane) - 1u));
			list[pos] = cell;
			W.dirty[cell] = 0;
			const int ix = cell % W.nx, iz = (cell / W.nx) % W.nz, iy = cell / (W.nx * W.nz);
			const int kRev[3] = {1, -1, 0};
			for (int i = 0; i < 27; ++i) { // common/include/common/Position.hpp:146-152
				const int dz = kRev[i % 3], dy = kRev[(i / 3) % 3], dx = kRev[i / 9];
				const int32_t slot = W.slots[cell_of(W, ix + dx, iy + dy, iz + dz)];
				nbr[(size_t)pos * 27 + i] = slot;
				slot_mark[slot] = 1;
			}
		}
		__syncthreads();
		if (tid == 0)
			s_base += total;
		__syncthreads();
	}
	if (tid == 0)
		count[0] = s_base, s_base = 0;
	__syncthreads();
	for (uint32_t s0 = 0; s0 < pool_cap; s0 += kEditThreads) {
		const uint32_t slot = s0 + tid;
		const bool take = slot < pool_cap && slot_mark[slot];
		const uint32_t bal = __ballot_sync(0xffffffffu, take);
		if (lane == 0)
			s_warp[warp] = __popc(bal);
		__syncthreads();
		uint32_t before = 0, total = 0;
		for (int w = 0; w < kEditThreads / 32; ++w) {
			before += w < warp ? s_warp[w] : 0;
			total += s_warp[w];
		}
		if (take) {
			slot_list[s_base + before + __popc(bal & ((1u << lane) - 1u))] = (int32_t)slot;
			slot_mark[slot] = 0;
		}
		__syncthreads();
		if (tid == 0)
			s_base += total;
		__syncthreads();
	}
	if (tid == 0)
		count[1] = s_base;
}

// Marks the listed chunks again (a remesh that did not fit its arena).
__global__ void k_remark(WorldDev W, const int32_t *list, uint32_t n) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n)
		W.dirty[list[i]] = 1;
}

} // namespace hc
