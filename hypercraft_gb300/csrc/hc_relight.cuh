// Window relight as a bit-sliced level cascade (one CTA, shared memory).
//
// The reference floods each light channel with a FIFO BFS inside the 62^3 window [-15, 47)^3 of a
// chunk (client/src/ChunkMeshTask.cpp:48-111, client/include/client/BlockLightAlgo.hpp:44-73):
// a cell of level L passes L-1 to a 6-neighbour n when L-1 >= 1, n lies in the window, n lets light
// through (transparency != opaque) and L-1 exceeds n's distance to the box [-1, 33)^3
// (IsBorderLightInterfere, BlockLightAlgo.hpp:32-42, Border = 14). The result is the least
// fixpoint of that rule above the seeds, which does not depend on visiting order. Writing S_t for
// the set of cells whose final level is >= t, the fixpoint satisfies
//     S_15 = seeds of level 15,
//     S_t  = S_{t+1}  |  seeds of level t  |  (pass & {dist < t} & dilate6(S_{t+1})),
// so fourteen 6-neighbour dilations of 62-bit row masks give every level exactly. A cell's light
// is the largest t with the cell in S_t. Only [-1, 32]^3 (what the mesher reads) is written out.
#pragma once
#include <cooperative_groups.h>

#include "hc_device.cuh"

namespace hc {

// How one chunk's work is shared by the CTAs of a thread-block cluster (a chunk meshed by several
// SMs, for latency). Face planes: CTA `rank` of `c` owns the slices axis * 33 + slice that are
// congruent to rank mod c, with both face directions of each. Relight window: CTA `rank` owns
// the window rows y in [rank * 62 / c, (rank + 1) * 62 / c). Every CTA stages the whole chunk.
struct Split {
	int c, rank;
	__device__ __forceinline__ int planes() const { return 2 * ((kSlices - rank + c - 1) / c); }
	__device__ __forceinline__ int plane(int j) const { return 2 * (rank + c * (j >> 1)) + (j & 1); }
	__device__ __forceinline__ int owner(int p) const { return (p >> 1) % c; }
	__device__ __forceinline__ int win_lo(int r) const { return r * kWin / c; }
	__device__ __forceinline__ int win_owner(int wy) const {
		int r = 0;
		while (r + 1 < c && win_lo(r + 1) <= wy)
			++r;
		return r;
	}
};

// Distance of one coordinate to [-1, 33) as IsBorderLightInterfere computes it.
__device__ __forceinline__ int axis_dist(int v) { return v < -1 ? -1 - v : (v >= 33 ? v - 33 : 0); }

// Cells of a window row whose distance to the box is below t, given rem = t - 1 - dy - dz >= 0.
__device__ __forceinline__ uint64_t dist_mask_rem(int rem) {
	int lo = 14 - rem, hi = 48 + rem;
	lo = lo < 0 ? 0 : lo;
	hi = hi > kWin - 1 ? kWin - 1 : hi;
	return ((~0ull) >> (63 - hi)) & ~((1ull << lo) - 1ull);
}

// The light of [-1, 32]^3 lives in the low byte of each staged cell (little-endian).
__device__ __forceinline__ uint8_t *light_bytes(Smem &S) { return reinterpret_cast<uint8_t *>(S.cell); }

// Writes level `t` into the light nibble of newly lit cells of row (wy, wz) inside [-1, 32]^3.
__device__ __forceinline__ void write_new(uint8_t *light, int wy, int wz, uint64_t bits, uint32_t t, int shift) {
	if (wy < 14 || wy > 47 || wz < 14 || wz > 47)
		return;
	bits &= 0x0000ffffffffc000ull; // window x in [14, 47]  <=>  x in [-1, 32]
	const int row = ((wy - 14) * kLt + (wz - 14)) * kLt;
	while (bits) {
		int b = __ffsll((long long)bits) - 1;
		bits &= bits - 1;
		light[2 * (row + b - 14)] |= (uint8_t)(t << shift);
	}
}

// Writes all 34 light bytes of a row inside [-1, 32]^3 from the level-15 sets.
__device__ __forceinline__ void write_row15(uint8_t *light, int wy, int wz, uint64_t sun, uint64_t torch) {
	if (wy < 14 || wy > 47 || wz < 14 || wz > 47)
		return;
	uint8_t *row = light + 2 * ((wy - 14) * kLt + (wz - 14)) * kLt;
	const uint64_t s = sun >> 14, t = torch >> 14;
#pragma unroll
	for (int i = 0; i < kLt; ++i)
		row[2 * i] = (uint8_t)((((s >> i) & 1u) ? 0x0fu : 0u) | (((t >> i) & 1u) ? 0xf0u : 0u));
}

// Seeds from the 27 chunks' bit planes: each window row joins three 32-bit chunk rows.
__device__ void seed_from_planes(Smem &S, int r_lo, int r_hi) {
	Relight &R = S.u.rl;
	for (int r = r_lo + threadIdx.x; r < r_hi; r += kThreads) {
		const int wy = r / kWin, wz = r - wy * kWin, y = wy - 15, z = wz - 15;
		const int prow = (z & 31) + 32 * (y & 31);
		uint32_t w[3][3], low = 0;
#pragma unroll
		for (int c = 0; c < 3; ++c) {
			const uint32_t *P = S.pln[nb_index(c * 32 - 1, y, z)];
#pragma unroll
			for (int pl = 0; pl < 3; ++pl)
				w[c][pl] = __ldg(P + pl * kPlaneWords + prow);
			low |= __ldg(P + kPlaneLowOff + (prow >> 5)) >> (prow & 31);
		}
		uint64_t v[3];
#pragma unroll
		for (int pl = 0; pl < 3; ++pl)
			v[pl] = (uint64_t)(w[0][pl] >> 17) | ((uint64_t)w[1][pl] << 15) | ((uint64_t)(w[2][pl] & 0x7fffu) << 47);
		R.pass[r] = v[kPlanePass];
		R.lit[r] = make_ulonglong2(v[kPlaneSun], v[kPlaneT15]);
		if (low & 1u)
			atomicOr(&R.low_rows[r >> 5], 1u << (r & 31));
		write_row15(light_bytes(S), wy, wz, v[kPlaneSun], v[kPlaneT15]);
	}
}

// Seeds from the blocks themselves (used when no planes are given), one warp per row.
__device__ void seed_from_blocks(Smem &S, const DevTables &T, int r_lo, int r_hi) {
	Relight &R = S.u.rl;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int r = r_lo + warp; r < r_hi; r += kWarps) {
		const int wy = r / kWin, wz = r - wy * kWin, y = wy - 15, z = wz - 15;
		uint64_t pass = 0, sun = 0, torch = 0;
		bool low = false;
#pragma unroll
		for (int half = 0; half < 2; ++half) {
			const int wx = lane + 32 * half, x = wx - 15;
			bool ip = false, sn = false, t15 = false;
			if (wx < kWin) {
				const DevClass &k = S.classes[__ldg(T.class_of + raw_at(S, x, y, z))];
				ip = k.flags & kFIndirect;
				sn = sunlit(S, x, y, z);
				t15 = k.light >= 15;
				low |= k.light > 0 && k.light < 15;
			}
			pass |= (uint64_t)__ballot_sync(0xffffffffu, ip) << (32 * half);
			sun |= (uint64_t)__ballot_sync(0xffffffffu, sn) << (32 * half);
			torch |= (uint64_t)__ballot_sync(0xffffffffu, t15) << (32 * half);
		}
		low = __any_sync(0xffffffffu, low);
		if (lane == 0) {
			R.pass[r] = pass;
			R.lit[r] = make_ulonglong2(sun, torch);
			if (low)
				atomicOr(&R.low_rows[r >> 5], 1u << (r & 31));
		}
	}
	__syncthreads();
	for (int r = r_lo + threadIdx.x; r < r_hi; r += kThreads) {
		const int wy = r / kWin, wz = r - wy * kWin;
		const ulonglong2 l = R.lit[r];
		write_row15(light_bytes(S), wy, wz, l.x, l.y);
	}
}

// Bit of row r in a row bitmap.
__device__ __forceinline__ bool row_bit(const uint32_t *m, int r) { return (m[r >> 5] >> (r & 31)) & 1u; }

// With sp.c > 1 the CTAs of a cluster share the window by rows (Split::win_lo): each seeds its
// rows and the row next to them on either side, runs the cascade on its own rows, and after every
// level takes the two neighbouring rows from the CTAs that own them (distributed shared memory);
// at the end each takes the light of [-1, 32]^3 the others computed. Every CTA of the cluster
// passes the same cluster barriers.
__device__ void relight_window(Smem &S, const DevTables &T, const Split &sp = Split{1, 0}) {
	namespace cg = cooperative_groups;
	Relight &R = S.u.rl;
	const int tid = threadIdx.x;
	const bool split = sp.c > 1;
	const int wlo = split ? sp.win_lo(sp.rank) : 0, whi = split ? sp.win_lo(sp.rank + 1) : kWin;
	const int seed_lo = (wlo > 0 ? wlo - 1 : 0) * kWin, seed_hi = (whi < kWin ? whi + 1 : kWin) * kWin;
	const int own_lo = wlo * kWin, own_hi = whi * kWin;
	for (int i = tid; i < kRowWords; i += kThreads)
		R.low_rows[i] = 0, R.changed[0][i] = 0, R.changed[1][i] = 0;
	__syncthreads();
	if (S.pln[26])
		seed_from_planes(S, seed_lo, seed_hi);
	else
		seed_from_blocks(S, T, seed_lo, seed_hi);
	__syncthreads();

	// A row can gain cells at level t only when it or one of its four neighbour rows changed at
	// level t + 1: otherwise its dilation is the one it already saw, while the distance mask only
	// shrinks. So after the first level only rows next to the last changes (the light front) and
	// rows holding emitters of the level are visited.
	constexpr int kRowsPerThread = (kWinRows + kThreads - 1) / kThreads;
	int rem0[kRowsPerThread]; // t - 1 - dist(y, z) = t + rem0
#pragma unroll
	for (int k = 0; k < kRowsPerThread; ++k) {
		const int r = own_lo + tid + k * kThreads;
		const int wy = r / kWin, wz = r - wy * kWin;
		rem0[k] = r < own_hi ? -1 - axis_dist(wy - 15) - axis_dist(wz - 15) : -1000;
	}
	uint8_t *light = light_bytes(S);
	for (int t = 14; t >= 1; --t) {
		const uint32_t *prev = R.changed[(t + 1) & 1];
		uint32_t *cur_chg = R.changed[t & 1];
		for (int i = tid; i < kRowWords; i += kThreads)
			cur_chg[i] = 0; // last read at level t + 1
		uint64_t ns[kRowsPerThread], nt[kRowsPerThread];
		uint32_t changed = 0;
#pragma unroll
		for (int k = 0; k < kRowsPerThread; ++k) {
			const int r = own_lo + tid + k * kThreads;
			const int rem = t + rem0[k];
			if (r >= own_hi)
				continue;
			const bool low = row_bit(R.low_rows, r);
			if (rem < 0 && !low)
				continue;
			const int wy = r / kWin, wz = r - wy * kWin;
			if (t < 14 && !low && !split) { // (split: the neighbour rows' changes are not tracked)
				const bool near = row_bit(prev, r) || (wz > 0 && row_bit(prev, r - 1)) ||
				                  (wz < kWin - 1 && row_bit(prev, r + 1)) || (wy > 0 && row_bit(prev, r - kWin)) ||
				                  (wy < kWin - 1 && row_bit(prev, r + kWin));
				if (!near)
					continue;
			}
			const ulonglong2 cur = R.lit[r];
			uint64_t s = cur.x, tt = cur.y;
			if (rem >= 0) {
				const uint64_t m = R.pass[r] & dist_mask_rem(rem);
				const uint64_t cs = m & ~cur.x, ct = m & ~cur.y; // cells that could still be lit
				if (cs | ct) {
					uint64_t ds = (cur.x << 1) | (cur.x >> 1), dt = (cur.y << 1) | (cur.y >> 1);
					if (wz > 0) {
						const ulonglong2 n = R.lit[r - 1];
						ds |= n.x, dt |= n.y;
					}
					if (wz < kWin - 1) {
						const ulonglong2 n = R.lit[r + 1];
						ds |= n.x, dt |= n.y;
					}
					if (wy > 0) {
						const ulonglong2 n = R.lit[r - kWin];
						ds |= n.x, dt |= n.y;
					}
					if (wy < kWin - 1) {
						const ulonglong2 n = R.lit[r + kWin];
						ds |= n.x, dt |= n.y;
					}
					s |= cs & ds;
					tt |= ct & dt;
				}
			}
			if (low) { // emitters of level t enter now
				const int y = wy - 15, z = wz - 15;
				for (int wx = 0; wx < kWin; ++wx)
					if (S.classes[__ldg(T.class_of + raw_at(S, wx - 15, y, z))].light == t)
						tt |= 1ull << wx;
			}
			if (s != cur.x || tt != cur.y) {
				ns[k] = s, nt[k] = tt;
				changed |= 1u << k;
			}
		}
		__syncthreads();
#pragma unroll
		for (int k = 0; k < kRowsPerThread; ++k) {
			if (!((changed >> k) & 1u))
				continue;
			const int r = own_lo + tid + k * kThreads;
			const int wy = r / kWin, wz = r - wy * kWin;
			const ulonglong2 cur = R.lit[r];
			R.lit[r] = make_ulonglong2(ns[k], nt[k]);
			atomicOr(&cur_chg[r >> 5], 1u << (r & 31));
			write_new(light, wy, wz, ns[k] & ~cur.x, (uint32_t)t, 0);
			write_new(light, wy, wz, nt[k] & ~cur.y, (uint32_t)t, 4);
		}
		__syncthreads();
		if (split) { // the rows next to this CTA's, as their owners left them at this level
			cg::cluster_group cl = cg::this_cluster();
			cl.sync();
			for (int i = tid; i < 2 * kWin; i += kThreads) {
				const int side = i / kWin, wz = i - side * kWin, wy = side ? whi : wlo - 1;
				if (wy >= 0 && wy < kWin)
					R.lit[wy * kWin + wz] = cl.map_shared_rank(&R.lit[0], sp.rank + (side ? 1 : -1))[wy * kWin + wz];
			}
			cl.sync();
		}
	}
	if (split) { // light of [-1, 32]^3 rows other CTAs own
		cg::cluster_group cl = cg::this_cluster();
		for (int i = tid; i < kLtCells; i += kThreads) {
			const int wy = i / (kLt * kLt) + 14;
			if (wy >= wlo && wy < whi)
				continue;
			light[2 * i] = (uint8_t)(cl.map_shared_rank(&S.cell[0], sp.win_owner(wy))[i] & 0xffu);
		}
		__syncthreads();
	}
}

// ------------------------------------------------------------------------------------ planes

// Bit planes of one 32-cell row (y, z) of a chunk: pass (transparency != opaque), sunlit
// (Chunk::GetSunlight), emitters of level 15, opaque full cubes and blank blocks, the row's class
// ids and its kLayer* summary bits (all but the z-row bits); returns whether the row holds an
// emitter of level 1..14. Uniform rows (one raw value) take one lookup.
__device__ __forceinline__ bool chunk_plane_row(const uint16_t *blk, const int8_t *hgt, const DevClass *classes,
                                                const uint8_t *class_of, int y, int z, uint32_t &pass, uint32_t &sun,
                                                uint32_t &t15, uint32_t cls[8], uint32_t &layer, uint32_t &oc,
                                                uint32_t &em) {
	const uint4 *row = reinterpret_cast<const uint4 *>(blk + (y * kChunk + z) * kChunk);
	uint4 q[4];
#pragma unroll
	for (int i = 0; i < 4; ++i)
		q[i] = __ldg(row + i);
	const uint32_t w0 = q[0].x;
	bool uniform = (w0 & 0xffffu) == (w0 >> 16);
#pragma unroll
	for (int i = 0; i < 4; ++i)
		uniform &= q[i].x == w0 && q[i].y == w0 && q[i].z == w0 && q[i].w == w0;
	bool low = false;
	pass = t15 = 0;
	if (uniform) {
		const uint32_t c = __ldg(class_of + (w0 & 0xffffu));
		const DevClass &k = classes[c];
		pass = (k.flags & kFIndirect) ? 0xffffffffu : 0u;
		t15 = k.light >= 15 ? 0xffffffffu : 0u;
		low = k.light > 0 && k.light < 15;
		layer = ((k.flags & kFEmpty) ? 0u : kLayerContent) |
		        ((k.flags & kFOpaqueCube) ? 0u : (kLayerOpen | kLayerOpenX0 | kLayerOpenX31)) |
		        ((k.mesh_meta & 3u) ? kLayerCustom : 0u);
		oc = (k.flags & kFOpaqueCube) ? 0xffffffffu : 0u;
		em = (k.flags & kFEmpty) ? 0xffffffffu : 0u;
#pragma unroll
		for (int i = 0; i < 8; ++i)
			cls[i] = c * 0x01010101u;
	} else {
#pragma unroll
		for (int i = 0; i < 8; ++i)
			cls[i] = 0;
		uint32_t custom = 0;
		oc = em = 0;
#pragma unroll
		for (int i = 0; i < 4; ++i) {
			const uint32_t ws[4] = {q[i].x, q[i].y, q[i].z, q[i].w};
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const uint32_t raw = (ws[j >> 1] >> (16 * (j & 1))) & 0xffffu;
				const uint32_t c = __ldg(class_of + raw);
				const DevClass &k = classes[c];
				const int x = 8 * i + j;
				pass |= (uint32_t)((k.flags & kFIndirect) != 0) << x;
				t15 |= (uint32_t)(k.light >= 15) << x;
				low |= k.light > 0 && k.light < 15;
				cls[x >> 2] |= c << (8 * (x & 3));
				em |= (uint32_t)((k.flags & kFEmpty) != 0) << x;
				oc |= (uint32_t)((k.flags & kFOpaqueCube) != 0) << x;
				custom |= k.mesh_meta & 3u;
			}
		}
		layer = (~em ? kLayerContent : 0u) | (~oc ? kLayerOpen : 0u) | ((oc & 1u) ? 0u : kLayerOpenX0) |
		        ((oc >> 31) ? 0u : kLayerOpenX31) | (custom ? kLayerCustom : 0u);
	}
	const uint4 *hr = reinterpret_cast<const uint4 *>(hgt + z * kChunk);
	const uint4 h[2] = {__ldg(hr), __ldg(hr + 1)};
	const uint32_t hw[8] = {h[0].x, h[0].y, h[0].z, h[0].w, h[1].x, h[1].y, h[1].z, h[1].w};
	sun = 0;
#pragma unroll
	for (int x = 0; x < 32; ++x) {
		const int8_t hv = (int8_t)((hw[x >> 2] >> (8 * (x & 3))) & 0xffu);
		sun |= (uint32_t)((uint32_t)y >= (uint32_t)(int32_t)hv) << x;
	}
	return low;
}

// Bit planes of chunks: one thread per 32-cell row, 32 rows (one flag word, one layer) per warp.
__device__ __forceinline__ void planes_row(const uint16_t *blk, const int8_t *hgt, const DevClass *cls_smem,
                                           const uint8_t *class_of, int r, uint32_t *out) {
	uint32_t pass, sun, t15, cls[8], layer, oc, em;
	const bool low = chunk_plane_row(blk, hgt, cls_smem, class_of, r >> 5, r & 31, pass, sun, t15, cls, layer, oc, em);
	out[kPlanePass * kPlaneWords + r] = pass;
	out[kPlaneOpaque * kPlaneWords + r] = oc;
	out[kPlaneEmpty * kPlaneWords + r] = em;
	out[kPlaneSun * kPlaneWords + r] = sun;
	out[kPlaneT15 * kPlaneWords + r] = t15;
	uint4 *co = reinterpret_cast<uint4 *>(out + kPlaneClassOff + 8 * r);
	co[0] = make_uint4(cls[0], cls[1], cls[2], cls[3]);
	co[1] = make_uint4(cls[4], cls[5], cls[6], cls[7]);
	const uint32_t lows = __ballot_sync(0xffffffffu, low);
	// the warp's rows are the layer y = r / 32, lane = z
	const uint32_t z = (uint32_t)(r & 31);
	const uint32_t sum = __reduce_or_sync(0xffffffffu, layer & (kLayerContent | kLayerOpen | kLayerOpenX0 | kLayerOpenX31 |
	                                                             kLayerCustom)) |
	                     (__reduce_or_sync(0xffffffffu, z == 0 ? layer : 0u) & kLayerOpen ? kLayerOpenZ0 : 0u) |
	                     (__reduce_or_sync(0xffffffffu, z == 31 ? layer : 0u) & kLayerOpen ? kLayerOpenZ31 : 0u);
	if ((threadIdx.x & 31) == 0) {
		out[kPlaneLowOff + (r >> 5)] = lows;
		out[kPlaneLayerOff + (r >> 5)] = sum;
	}
}


// ------------------------------------------------------------------------------- batch light pass
//
// The batched form lights all chunks of a batch at once instead of relighting a 62^3 window per
// chunk (which covers each cell about seven times). On the box [-1, 33)^3 of a chunk the window's
// fixpoint equals the fixpoint of the same rule over every chunk of the batch without the window
// and border bounds: a light path that ends in the box at level >= 1 only visits cells whose level
// exceeds their distance to the box, and level <= 15 keeps such cells inside [-15, 47)^3, which
// lies inside the 27 chunks the batch holds for that chunk. So with S_t = {cells of level >= t}
// over the batch,
//     S_15 = seeds of level 15,   S_t = S_{t+1} | seeds of level t | (pass & dilate6(S_{t+1})),
// fifteen passes over all chunks give every level; face neighbours missing from the batch count as
// dark (they lie outside every meshed chunk's window).

constexpr int kLevels = 15;
constexpr size_t kLevelSlotWords = (size_t)2 * kLevels * kPlaneWords; // per chunk: 2 channels x 15 levels
constexpr size_t kEdgeSlotWords = (size_t)2 * kLevels * 2 * 32;       // per chunk: x = 0 and x = 31 bits
constexpr int kLightWarps = 4;       // warps per block, one chunk channel each
constexpr int kLightThreads = 32 * kLightWarps;
constexpr int kLightBlocksPerSM = 12; // register bound: 40 per thread

struct LightPass {
	const int32_t *slots;   // batch chunk -> pool slot
	const int32_t *nb6;     // batch chunk -> face neighbours (batch chunk or -1): -x, +x, -y, +y, -z, +z
	const uint32_t *planes; // pool planes (pass, sun, level-15 emitters, low-emitter rows)
	const uint16_t *blocks; // pool blocks (rows with emitters below 15)
	uint32_t *levels;       // batch chunk -> channel -> level t at plane t - 1 -> 1024 rows
	uint32_t *edges;        // batch chunk -> channel -> level -> {bit x = 0, bit x = 31} of every row
	uint32_t *flags;        // batch chunk -> channel -> kFlag* bits of its level planes
	uint32_t *near;         // batch chunk -> channel -> bit t - 1: some face neighbour (or the chunk) has a
	                        // non-empty level t + 1 (set by those chunks; cleared before the pass)
	uint32_t n;             // batch chunks
};

// Per batch chunk and channel, which level planes are uniform: bit t - 1 = level t is empty, bit
// 16 + t - 1 = level t is full. A uniform plane below level 15 whose value follows from level t + 1
// (full stays full; empty stays empty when the six face neighbours are empty and no emitter seeds
// it) is neither computed nor stored: every reader takes its value from these bits. Bit 15 of the
// torch word: the chunk holds emitters below level 15.
enum : uint32_t { kFlagFull = 16, kFlagLowEmitters = 1u << 15 };
__device__ __forceinline__ bool level_empty(uint32_t f, int t) { return (f >> (t - 1)) & 1u; }
__device__ __forceinline__ bool level_full(uint32_t f, int t) { return (f >> (kFlagFull + t - 1)) & 1u; }
// The word of a level plane row (or edge word) from its chunk's flags, or loaded when not uniform.
__device__ __forceinline__ uint32_t level_word(uint32_t f, int t, const uint32_t *p) {
	return level_empty(f, t) ? 0u : (level_full(f, t) ? 0xffffffffu : __ldg(p));
}

__device__ __forceinline__ const uint32_t *level_plane(const LightPass &L, int i, int c, int t) {
	return L.levels + (size_t)i * kLevelSlotWords + (size_t)(c * kLevels + t - 1) * kPlaneWords;
}
__device__ __forceinline__ const uint32_t *level_edges(const LightPass &L, int i, int c, int t) {
	return L.edges + (size_t)i * kEdgeSlotWords + (size_t)(c * kLevels + t - 1) * 64;
}

__device__ __forceinline__ uint32_t mux(uint32_t c, uint32_t a, uint32_t b) { return (c & a) | (~c & b); }

// 4-bit light of the 32 cells of a row from its 15 nested level words (s[t - 1] = S_t).
__device__ __forceinline__ void level_bits(const uint32_t *s, uint32_t b[4]) {
	b[3] = s[7];
	b[2] = mux(b[3], s[11], s[3]);
	b[1] = mux(b[3], mux(b[2], s[13], s[9]), mux(b[2], s[5], s[1]));
	b[0] = mux(b[3], mux(b[2], mux(b[1], s[14], s[12]), mux(b[1], s[10], s[8])),
	           mux(b[2], mux(b[1], s[6], s[4]), mux(b[1], s[2], s[0])));
}

// Level t of every batch chunk, one warp per chunk and channel (lane = z): the warp walks the
// chunk's 32 y layers, keeping the level t + 1 rows of layers y - 1, y and y + 1 in registers, and
// dilates each layer with shifts (x), shuffles (z) and the neighbouring layers (y). The face
// neighbours' touching rows and edge bits are loaded once, one word per lane. Also writes the row
// edge bits that the x neighbours read at the next level, and the plane's uniform bits
// (LightPass::flags). A channel whose level follows from level t + 1 without computing (see kFlag*)
// is skipped: a chunk of sunlit air far from any emitter costs one flag word per level and channel.
// No block barrier: the warps of a block are independent.
__global__ void __launch_bounds__(kLightThreads, kLightBlocksPerSM) k_light_level(LightPass L, DevTables T, int t) {
	constexpr uint32_t kAll = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	const uint32_t w = blockIdx.x * kLightWarps + (threadIdx.x >> 5);
	const uint32_t i = w >> 1;
	const int c = (int)(w & 1u); // 0: sun, 1: torch
	if (i >= L.n) // the whole warp
		return;
	// lanes 0-5: the face neighbours; lane 6: the pool slot; lane 8: the channel's flags; lane 10:
	// its near bits (flags and near bits from level t + 1)
	int32_t v1 = -1;
	if (lane < 6)
		v1 = __ldg(L.nb6 + 6 * (size_t)i + lane);
	else if (lane == 6)
		v1 = __ldg(L.slots + i);
	else if (t < kLevels && lane == 8)
		v1 = (int32_t)__ldg(L.flags + 2 * (size_t)i + c);
	else if (t < kLevels && lane == 10)
		v1 = (int32_t)__ldg(L.near + 2 * (size_t)i + c);
	const int slot = __shfl_sync(kAll, v1, 6);
	const int near_nb = lane < 6 ? v1 : (int)i; // lanes 0-6: the chunks whose near bits this one sets
	const uint32_t *P = L.planes + (size_t)slot * kPlaneStride;
	uint32_t *const lev = L.levels + (size_t)i * kLevelSlotWords + (size_t)c * kLevels * kPlaneWords;
	uint32_t *const edg = L.edges + (size_t)i * kEdgeSlotWords + (size_t)c * kLevels * 64;
	uint32_t *const flag = L.flags + 2 * (size_t)i + c;
	if (t == kLevels) { // the seeds: sunlit cells, emitters of level 15 (uniform planes are not stored)
		const uint32_t *seed = P + (c ? kPlaneT15 : kPlaneSun) * kPlaneWords;
		bool any = false, all = true;
#pragma unroll 8
		for (int y = 0; y < 32; ++y) {
			const uint32_t s = __ldg(seed + y * 32 + lane);
			any |= s != 0, all &= s == kAll;
		}
		const bool a = __any_sync(kAll, any), f = __all_sync(kAll, all);
		uint32_t fl = (a ? 0u : 1u << (kLevels - 1)) | (f ? 1u << (kFlagFull + kLevels - 1) : 0u);
		if (c == 1)
			fl |= __any_sync(kAll, __ldg(P + kPlaneLowOff + lane) != 0) ? kFlagLowEmitters : 0u;
		if (a && !f) { // the rows again (in L1 now), stored with their edge bits
			uint32_t elo = 0u, ehi = 0u;
			uint32_t *out = lev + (size_t)(kLevels - 1) * kPlaneWords;
#pragma unroll 8
			for (int y = 0; y < 32; ++y) {
				const uint32_t s = __ldg(seed + y * 32 + lane);
				out[y * 32 + lane] = s;
				const uint32_t lo = __ballot_sync(kAll, s & 1u), hi = __ballot_sync(kAll, s >> 31);
				if (lane == y)
					elo = lo, ehi = hi;
			}
			uint32_t *e = edg + (size_t)(kLevels - 1) * 64;
			e[lane] = elo;
			e[32 + lane] = ehi;
		}
		if (lane == 0)
			*flag = fl;
		if (a && lane < 7 && near_nb >= 0) // a non-empty level 15 may light the chunk and its face neighbours at level 14
			atomicOr(L.near + 2 * (size_t)near_nb + c, 1u << (kLevels - 2));
		return;
	}
	const uint32_t own = (uint32_t)__shfl_sync(kAll, v1, 8), nr = (uint32_t)__shfl_sync(kAll, v1, 10);
	// a channel that follows from level t + 1 without computing: full stays full; empty stays empty
	// when no face neighbour had light at level t + 1 and no emitter seeds level t
	const bool full = level_full(own, t + 1);
	if (full || (level_empty(own, t + 1) && !((nr >> (t - 1)) & 1u) && !(c == 1 && (own & kFlagLowEmitters)))) {
		if (lane == 0)
			atomicOr(flag, full ? 1u << (kFlagFull + t - 1) : 1u << (t - 1));
		// a full plane at level t (it stays full) lights the chunk and its face neighbours at level t - 1
		if (full && t > 1 && lane < 7 && near_nb >= 0)
			atomicOr(L.near + 2 * (size_t)near_nb + c, 1u << (t - 2));
		return;
	}
	// lanes 0-5: the face neighbours' level t + 1 flags (a missing neighbour is dark: empty)
	const uint32_t nfl = lane < 6 && v1 >= 0 ? __ldg(L.flags + 2 * (size_t)v1 + c) : 0xffffu;
	// lane k: x = -1 bits over z of layer k, x = 32 bits, the y = -1 and y = 32 rows at z = k, the
	// z = -1 and z = 32 rows of layer k
	uint32_t side[6];
#pragma unroll
	for (int f = 0; f < 6; ++f) {
		const int nb = __shfl_sync(kAll, v1, f);
		const uint32_t fl = __shfl_sync(kAll, nfl, f);
		side[f] = 0u;
		if (nb < 0)
			continue;
		const uint32_t *e = L.edges + (size_t)nb * kEdgeSlotWords + (size_t)(c * kLevels + t) * 64;
		const uint32_t *p = L.levels + (size_t)nb * kLevelSlotWords + (size_t)(c * kLevels + t) * kPlaneWords;
		const int off = f == 0 ? 32 + lane : f == 1 ? lane : f == 2 ? 31 * 32 + lane : f == 3 ? lane
		              : f == 4 ? lane * 32 + 31 : lane * 32;
		side[f] = level_word(fl, t + 1, (f < 2 ? e : p) + off);
	}
	// the chunk's own level t + 1 rows: stored, or a constant (a computed channel's level t + 1 is
	// stored or empty)
	const uint32_t *src = lev + (size_t)t * kPlaneWords;
	const bool stored = !level_empty(own, t + 1);
	const uint32_t lows = c == 1 ? __ldg(P + kPlaneLowOff + lane) : 0u; // lane y: low-emitter rows of layer y
	uint32_t up = side[2], me = stored ? __ldg(src + lane) : 0u;
	uint32_t elo = 0u, ehi = 0u, any = 0u, all = kAll;
	uint32_t *out = lev + (size_t)(t - 1) * kPlaneWords;
	constexpr int kBatch = 8; // layers whose rows are requested together
	for (int y0 = 0; y0 < 32; y0 += kBatch) {
		uint32_t pass[kBatch], next[kBatch];
#pragma unroll
		for (int j = 0; j < kBatch; ++j) {
			const int y = y0 + j;
			pass[j] = __ldg(P + kPlanePass * kPlaneWords + y * 32 + lane);
			next[j] = y < 31 ? (stored ? __ldg(src + (y + 1) * 32 + lane) : 0u) : side[3];
		}
#pragma unroll
		for (int j = 0; j < kBatch; ++j) {
			const int y = y0 + j;
			const uint32_t m = me, dn = next[j];
			const uint32_t xm = __shfl_sync(kAll, side[0], y), xp = __shfl_sync(kAll, side[1], y);
			const uint32_t zm = __shfl_sync(kAll, side[4], y), zp = __shfl_sync(kAll, side[5], y);
			const uint32_t zl = __shfl_up_sync(kAll, m, 1), zr = __shfl_down_sync(kAll, m, 1);
			uint32_t d = (m << 1) | (m >> 1) | up | dn;
			d |= (xm >> lane) & 1u;
			d |= ((xp >> lane) & 1u) << 31;
			d |= lane > 0 ? zl : zm;
			d |= lane < 31 ? zr : zp;
			uint32_t s = m | (pass[j] & d);
			// emitters below level 15: each row of the layer that holds some, by the whole warp
			for (uint32_t rows = __shfl_sync(kAll, lows, y); rows; rows &= rows - 1) {
				const int z = __ffs(rows) - 1;
				const uint16_t b = __ldg(L.blocks + (size_t)slot * 32768 + (y * 32 + z) * 32 + lane);
				const uint32_t seeded = __ballot_sync(kAll, T.classes[T.class_of[b]].light >= t);
				if (lane == z)
					s |= seeded;
			}
			any |= s, all &= s;
			out[y * 32 + lane] = s;
			const uint32_t lo = __ballot_sync(kAll, s & 1u), hi = __ballot_sync(kAll, s >> 31);
			if (lane == y)
				elo = lo, ehi = hi;
			up = m;
			me = dn;
		}
	}
	// a computed plane that came out uniform is flagged too (it is stored as well); a non-empty one
	// lights the chunk and its face neighbours at level t - 1
	uint32_t *e = edg + (size_t)(t - 1) * 64;
	e[lane] = elo;
	e[32 + lane] = ehi;
	const bool a = __any_sync(kAll, any != 0), f = __all_sync(kAll, all == kAll);
	if (lane == 0 && (!a || f))
		atomicOr(flag, !a ? 1u << (t - 1) : 1u << (kFlagFull + t - 1));
	if (a && t > 1 && lane < 7 && near_nb >= 0)
		atomicOr(L.near + 2 * (size_t)near_nb + c, 1u << (t - 2));
}

// Light bytes of the eight cells x = 8g .. 8g + 7 from the eight digit planes of a row (sun digits
// 0-3, then torch digits 0-3): byte g of every plane gathered into one 8 x 8 bit matrix (row k =
// plane k), transposed so that byte j holds bit x = 8g + j of every plane, by the three-step 8 x 8
// bit-matrix transpose of Warren, Hacker's Delight, section 7-3.
__device__ __forceinline__ uint64_t light_bytes8(const uint32_t w[8], int g) {
	const uint32_t sel = (uint32_t)g | ((uint32_t)(g + 4) << 4);
	const uint32_t lo = __byte_perm(__byte_perm(w[0], w[1], sel), __byte_perm(w[2], w[3], sel), 0x5410);
	const uint32_t hi = __byte_perm(__byte_perm(w[4], w[5], sel), __byte_perm(w[6], w[7], sel), 0x5410);
	uint64_t x = ((uint64_t)hi << 32) | lo, t;
	t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
	x ^= t ^ (t << 7);
	t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
	x ^= t ^ (t << 14);
	t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
	x ^= t ^ (t << 28);
	return x;
}

// The light-pass decode of one item of light_from_levels: item it < 34 * 34 is row (y, z) =
// (it / 34 - 1, it % 34 - 1), x in [0, 32), returned as 32 light bytes in v[0..3] (true); the others
// are the x = -1 and x = 32 edge pieces, written straight into the low bytes of their cells (false).
__device__ __forceinline__ bool light_item(Smem &S, int it, uint64_t v[4]) {
	constexpr int kRowItems = kLt * kLt;
	uint8_t *light = light_bytes(S);
	const uint32_t *src;
	int stride, nb;
	int x = 0, y, zc = 1, z0 = 0;
	if (it < kRowItems) {
		y = it / kLt - 1;
		const int z = it % kLt - 1;
		nb = nb_index(0, y, z);
		src = S.lvl[nb] + (y & 31) * 32 + (z & 31);
		stride = kPlaneWords;
	} else {
		const int k = it - kRowItems, side = k / (kLt * 3), rem = k - side * (kLt * 3);
		y = rem / 3 - 1, zc = rem % 3;
		x = side ? kChunk : -1, z0 = zc == 0 ? -1 : (zc == 1 ? 0 : kChunk);
		nb = nb_index(x, y, z0);
		src = S.edg[nb] + (side ? 0 : 32) + (y & 31); // x = 0 or x = 31 bits over z
		stride = 64;
	}
	uint32_t b[2][4];
#pragma unroll
	for (int c = 0; c < 2; ++c) {
		const uint32_t fl = S.lfl[nb][c]; // uniform planes are not stored
		uint32_t lv[kLevels];
#pragma unroll
		for (int u = 0; u < kLevels; ++u)
			lv[u] = level_word(fl, u + 1, src + (size_t)(c * kLevels + u) * stride);
		level_bits(lv, b[c]);
	}
	const uint32_t w[8] = {b[0][0], b[0][1], b[0][2], b[0][3], b[1][0], b[1][1], b[1][2], b[1][3]};
	if (it < kRowItems) {
#pragma unroll
		for (int g = 0; g < 4; ++g)
			v[g] = light_bytes8(w, g);
		return true;
	}
	if (zc == 1) { // 32 cells along z
		uint8_t *dst = light + 2 * lt_index(x, y, 0);
#pragma unroll
		for (int g = 0; g < 4; ++g) {
			const uint64_t q = light_bytes8(w, g);
#pragma unroll
			for (int j = 0; j < 8; ++j)
				dst[2 * kLt * (8 * g + j)] = (uint8_t)(q >> (8 * j));
		}
	} else { // the corner cell z = -1 (bit 31 of the -z chunk) or z = 32 (bit 0 of the +z chunk)
		const int bz = z0 & 31;
		uint32_t q = 0;
#pragma unroll
		for (int bit = 0; bit < 8; ++bit)
			q |= ((w[bit] >> bz) & 1u) << bit;
		light[2 * lt_index(x, y, z0)] = (uint8_t)q;
	}
	return false;
}

// Light bytes of the chunk's own row (y, z), both in [0, 32), from its 15 nested level planes per
// channel: uniform planes as constants, the planes staged in shared memory (`staged`, slot
// S.lvl_slot[plane] of 1,024 words each) from there, the others from global memory.
__device__ __forceinline__ void light_own_row(const Smem &S, int y, int z, const uint32_t *staged, uint64_t v[4]) {
	const int w = y * 32 + z;
	uint32_t b[2][4];
#pragma unroll
	for (int c = 0; c < 2; ++c) {
		const uint32_t fl = S.lfl[26][c];
		uint32_t lv[kLevels];
#pragma unroll
		for (int u = 0; u < kLevels; ++u) {
			const int slot = S.lvl_slot[c * kLevels + u];
			lv[u] = level_empty(fl, u + 1) ? 0u
			        : level_full(fl, u + 1) ? 0xffffffffu
			        : slot >= 0 ? staged[slot * kPlaneWords + w]
			                    : __ldg(S.lvl[26] + (size_t)(c * kLevels + u) * kPlaneWords + w);
		}
		level_bits(lv, b[c]);
	}
	const uint32_t q[8] = {b[0][0], b[0][1], b[0][2], b[0][3], b[1][0], b[1][1], b[1][2], b[1][3]};
#pragma unroll
	for (int g = 0; g < 4; ++g)
		v[g] = light_bytes8(q, g);
}

// Writes the 32 cells x in [0, 32) of row item `row` (34 * (y + 1) + z + 1): light bytes from v,
// class ids from the 32 bytes at `cls`. Cell 0 and cell 31 as halves, cells 1-30 as aligned pairs.
__device__ __forceinline__ void write_row_cells(Smem &S, int row, const uint64_t v[4], const uint8_t *cls) {
	uint16_t *c = S.cell + row * kCls + 1;
	const uint4 k0 = *reinterpret_cast<const uint4 *>(cls), k1 = *reinterpret_cast<const uint4 *>(cls + 16);
	const uint32_t kw[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
	const uint32_t lw[8] = {(uint32_t)v[0], (uint32_t)(v[0] >> 32), (uint32_t)v[1], (uint32_t)(v[1] >> 32),
	                        (uint32_t)v[2], (uint32_t)(v[2] >> 32), (uint32_t)v[3], (uint32_t)(v[3] >> 32)};
	// cell i = light byte i | class byte i << 8: the low and high byte pairs of each 4-cell group
	uint32_t pair[16];
#pragma unroll
	for (int q = 0; q < 8; ++q) {
		pair[2 * q] = __byte_perm(lw[q], kw[q], 0x5140);     // cells 4q, 4q + 1
		pair[2 * q + 1] = __byte_perm(lw[q], kw[q], 0x7362); // cells 4q + 2, 4q + 3
	}
	c[0] = (uint16_t)pair[0];
	uint32_t *c2 = reinterpret_cast<uint32_t *>(c + 1);
#pragma unroll
	for (int i = 0; i < 15; ++i) // cells 2i + 1, 2i + 2
		c2[i] = __byte_perm(pair[i], pair[i + 1], 0x5432);
	c[31] = (uint16_t)(pair[15] >> 16);
}

// Light of [-1, 32]^3 from the batch light pass (instead of relight_window), decoded from the 15
// nested level planes per channel into the low byte of every staged cell: a cell's light is the
// number of levels that hold it, read as four binary digits by level_bits. Cells x in [0, 32) of
// each row come from the level words of the row's chunk; x = -1 and x = 32 from the x neighbours'
// edge bits, 32 rows (z) per word.
__device__ void light_from_levels(Smem &S) {
	uint8_t *light = light_bytes(S);
	// one item per thread and round: the 34 x 34 rows (x in [0, 32)), then the 2 x 34 x 3 edge
	// pieces (x = -1 or 32; z = -1, [0, 32) or 32), so that both kinds share the second round
	constexpr int kRowItems = kLt * kLt, kItems = kRowItems + 2 * kLt * 3;
	for (int it = threadIdx.x; it < kItems; it += kThreads) {
		const uint32_t *src;
		int stride, nb;
		int x = 0, y, zc = 1, z0 = 0;
		if (it < kRowItems) {
			y = it / kLt - 1;
			const int z = it % kLt - 1;
			nb = nb_index(0, y, z);
			src = S.lvl[nb] + (y & 31) * 32 + (z & 31);
			stride = kPlaneWords;
		} else {
			const int k = it - kRowItems, side = k / (kLt * 3), rem = k - side * (kLt * 3);
			y = rem / 3 - 1, zc = rem % 3;
			x = side ? kChunk : -1, z0 = zc == 0 ? -1 : (zc == 1 ? 0 : kChunk);
			nb = nb_index(x, y, z0);
			src = S.edg[nb] + (side ? 0 : 32) + (y & 31); // x = 0 or x = 31 bits over z
			stride = 64;
		}
		uint32_t b[2][4];
#pragma unroll
		for (int c = 0; c < 2; ++c) {
			const uint32_t fl = S.lfl[nb][c]; // uniform planes are not stored
			uint32_t lv[kLevels];
#pragma unroll
			for (int u = 0; u < kLevels; ++u)
				lv[u] = level_word(fl, u + 1, src + (size_t)(c * kLevels + u) * stride);
			level_bits(lv, b[c]);
		}
		const uint32_t w[8] = {b[0][0], b[0][1], b[0][2], b[0][3], b[1][0], b[1][1], b[1][2], b[1][3]};
		if (zc == 1) { // 32 cells along x (a row) or along z (an x edge)
			uint8_t *dst = it < kRowItems ? light + 2 * (it * kLt + 1) : light + 2 * lt_index(x, y, 0);
			const int step = it < kRowItems ? 2 : 2 * kLt;
#pragma unroll
			for (int g = 0; g < 4; ++g) {
				const uint64_t v = light_bytes8(w, g);
#pragma unroll
				for (int j = 0; j < 8; ++j)
					dst[step * (8 * g + j)] = (uint8_t)(v >> (8 * j));
			}
		} else { // the corner cell z = -1 (bit 31 of the -z chunk) or z = 32 (bit 0 of the +z chunk)
			const int bz = z0 & 31;
			uint32_t v = 0;
#pragma unroll
			for (int bit = 0; bit < 8; ++bit)
				v |= ((w[bit] >> bz) & 1u) << bit;
			light[2 * lt_index(x, y, z0)] = (uint8_t)v;
		}
	}
}

} // namespace hc
