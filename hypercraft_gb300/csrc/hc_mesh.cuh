// Chunk mesher: one CTA per chunk, everything staged in shared memory.
//
// Reproduces BlockMeshAlgo<Config{int8, [0,32)^3, YZX}>::Generate
// (client/include/client/BlockMeshAlgo.hpp:494-521) exactly:
//   * custom meshes first, blocks in (y, z, x) order, faces in list order (198-306);
//   * then axes x, y, z; per axis slices 0..32; per slice the +dir then the -dir face plane
//     (308-482), each plane merged greedily: width along V first, then height along U,
//     scanning u-major (345-477);
//   * two vertex streams (opaque / transparent pass); a stream's mesh is closed when four more
//     vertices would exceed 65,535, and closed meshes are emitted in closing order, followed by
//     the open opaque and the open transparent mesh (272-279, 396-403, 515-518).
//
// Parallel form. A plane's cells are keyed by (texture, Light4); the greedy merge only ever
// compares a cell with its right and lower neighbour (equality is transitive), so each plane is
// reduced to four 32x32 bit masks: visible, equal-to-right, equal-to-below and transparent-pass.
// Warps build them with ballots and then run the exact sequential greedy scan on the masks with
// word operations, one warp per plane. Counts per (stream, segment) are prefix-summed in
// output order, which gives every quad its final stream index k before anything is written, so
// all quads are written in parallel straight to their reference positions.
#pragma once
#include <cooperative_groups.h>

#include "hc_relight.cuh"

namespace hc {


// Next index of a per-plane phase for the calling warp (all lanes get it): warps take planes as
// they finish the previous one, so a phase ends when the work does, not when the unluckiest warp's
// fixed share does.
__device__ __forceinline__ int claim(uint32_t *counter) {
	int j = 0;
	if ((threadIdx.x & 31) == 0)
		j = (int)atomicAdd(counter, 1u);
	return __shfl_sync(0xffffffffu, j, 0);
}
enum : int { kClaimKeys = 13, kClaimLone = 14, kMine = 15 }; // S.misc counters

// Orders the face planes by falling weight class (visible faces and complex candidates; class =
// the weight's bit length, so the weights of a class are within a factor of two) into S.order, so
// that the key pass takes the heaviest planes first and its last planes are light ones
// (longest-processing-time order, to a factor of two), planes of a class in plane order. A counting
// sort: every thread of the first warps takes one plane and finds its rank from per-warp class
// counts (warp match), so the order is the same on every run and in every CTA of a cluster (they
// compute it from the same masks). Weights sit in seg_base[0], the count tables in seg_base[1],
// both unused until the scan. Returns how many planes have any face: the rest are left out of the
// key pass (their counts stay 0; their owner is CTA 0).
__device__ int order_planes(Smem &S) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	constexpr int kClasses = 12, kOrderWarps = (kPlanes + 31) / 32; // weight <= 1,024: bit length <= 11
	static_assert(2 * kClasses * kOrderWarps <= kSegments + 1, "count tables fit in seg_base[1]");
	uint32_t *weight = &S.seg_base[0][0];
	uint32_t *cnt = &S.seg_base[1][0], *base = cnt + kClasses * kOrderWarps; // [warp][class]
	for (int p = warp; p < kPlanes; p += kWarps) {
		const uint32_t w = __reduce_add_sync(0xffffffffu, __popc(S.u.masks[p][lane][0] | S.u.masks[p][lane][1]));
		if (lane == 0)
			weight[p] = w;
	}
	if (threadIdx.x < kClasses * kOrderWarps)
		cnt[threadIdx.x] = 0;
	__syncthreads();
	const int p = threadIdx.x;
	uint32_t cls = 0, before = 0; // this plane's class, and planes of its class earlier in its warp
	if (warp < kOrderWarps) {
		const uint32_t w = p < kPlanes ? weight[p] : 0u;
		cls = w ? 32u - __clz(w) : 0u;
		const uint32_t peers = __match_any_sync(0xffffffffu, p < kPlanes ? cls : 0xffu);
		before = __popc(peers & ((1u << lane) - 1u));
		if (p < kPlanes && before == 0)
			cnt[warp * kClasses + cls] = __popc(peers);
	}
	__syncthreads();
	if (warp == 0) { // lane = class: planes in heavier classes, then in earlier warps of the same class
		uint32_t tot = 0;
		if (lane < kClasses)
			for (int k = 0; k < kOrderWarps; ++k)
				tot += cnt[k * kClasses + lane];
		uint32_t heavier = tot; // becomes the sum over classes >= lane, then > lane
#pragma unroll
		for (int d = 1; d < 16; d <<= 1) {
			const uint32_t o = __shfl_down_sync(0xffffffffu, heavier, d);
			if (lane + d < kClasses)
				heavier += o;
		}
		uint32_t run = heavier - tot;
		if (lane < kClasses)
			for (int k = 0; k < kOrderWarps; ++k) {
				base[k * kClasses + lane] = run;
				run += cnt[k * kClasses + lane];
			}
	}
	__syncthreads();
	if (warp < kOrderWarps && p < kPlanes) {
		S.order[base[warp * kClasses + cls] + before] = (uint8_t)p;
		if (weight[p] == 0)
			S.plane_owner[p] = 0;
	}
	return __syncthreads_count(threadIdx.x < kPlanes && weight[threadIdx.x] > 0);
}

// Next face plane for the calling warp's key pass. In a cluster the planes are taken from one
// counter in CTA 0, so a heavy plane does not hold up a CTA with a fixed share; the taker records
// the plane as its own (count and emission run where its masks are) and in CTA 0's owner table.
__device__ __forceinline__ int claim_plane(Smem &S, const Split &sp, int live) {
	int p = 0;
	if ((threadIdx.x & 31) == 0) {
		if (sp.c > 1) {
			cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
			p = (int)atomicAdd(cl.map_shared_rank(&S.misc[kClaimKeys], 0), 1u);
			p = p < live ? (int)S.order[p] : kPlanes;
			if (p < kPlanes) {
				cl.map_shared_rank(&S.plane_owner[0], 0)[p] = (uint8_t)sp.rank;
			}
		} else {
			p = (int)atomicAdd(&S.misc[kClaimKeys], 1u);
			p = p < live ? (int)S.order[p] : kPlanes;
		}
		if (p < kPlanes)
			S.mine[atomicAdd(&S.misc[kMine], 1u)] = (uint8_t)p;
	}
	return __shfl_sync(0xffffffffu, p, 0);
}

struct Emit {
	uint2 *verts;
	uint16_t *idx;
	unsigned long long q0; // first quad of this chunk in the arena
	uint32_t qo;           // opaque quads (the transparent stream starts after them)
};

// Grows the bounding box of mesh (st, m) by [mn, mx]; one thread.
__device__ __forceinline__ void aabb_add(Smem &S, int st, uint32_t m, const uint32_t mn[3], const uint32_t mx[3]) {
	uint32_t *bb = S.aabb[st][m];
	atomicMin(bb + 0, mn[0]), atomicMin(bb + 1, mn[1]), atomicMin(bb + 2, mn[2]);
	atomicMax(bb + 3, mx[0]), atomicMax(bb + 4, mx[1]), atomicMax(bb + 5, mx[2]);
}

// A warp's running box of one mesh (key = stream << 16 | mesh; every lane holds the box of its own
// quads of that mesh): the emission grows it quad by quad in registers and adds it to the mesh's
// box in shared memory (a warp reduction and six atomics) only when the warp moves on to another
// mesh, and once at the end, instead of once per round of 32 quads.
struct BoxAcc {
	uint32_t key = 0xffffffffu;
	uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
};

// Adds the running box to its mesh's box (all lanes call it).
__device__ __forceinline__ void box_flush(Smem &S, BoxAcc &b) {
	if (b.key == 0xffffffffu)
		return;
	uint32_t r[6];
#pragma unroll
	for (int c = 0; c < 3; ++c) {
		r[c] = __reduce_min_sync(0xffffffffu, b.mn[c]);
		r[3 + c] = __reduce_max_sync(0xffffffffu, b.mx[c]);
		b.mn[c] = 0xffffffffu, b.mx[c] = 0u;
	}
	if ((threadIdx.x & 31) == 0)
		aabb_add(S, (int)(b.key >> 16), b.key & 0xffffu, r, r + 3);
	b.key = 0xffffffffu;
}

// Grows the boxes by one round of quads (all lanes call it; `valid` lanes carry a quad of mesh
// (st, m) spanning [mn, mx]). The quads of the first valid lane's mesh go into the running box; a
// lane of another mesh (a round that crosses a mesh boundary) adds its quad directly.
__device__ __forceinline__ void box_add_warp(Smem &S, BoxAcc &b, bool valid, int st, uint32_t m, const uint32_t mn[3],
                                             const uint32_t mx[3]) {
	const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
	if (!vmask)
		return;
	const uint32_t key = ((uint32_t)st << 16) | m;
	const uint32_t lkey = __shfl_sync(0xffffffffu, key, __ffs(vmask) - 1);
	if (lkey != b.key) {
		box_flush(S, b);
		b.key = lkey;
	}
	if (valid && key == lkey) {
#pragma unroll
		for (int c = 0; c < 3; ++c) {
			b.mn[c] = min(b.mn[c], mn[c]);
			b.mx[c] = max(b.mx[c], mx[c]);
		}
	} else if (valid) {
		aabb_add(S, st, m, mn, mx);
	}
}

// Writes quad k of stream st (all-stream index g): 4 vertices, 6 indices, and the trigger of the
// mesh it closes. The caller grows the mesh's box.
__device__ __forceinline__ void put_quad(Smem &S, const Emit &E, int st, uint32_t k, uint32_t g, const uint2 v[4], bool flip) {
	const unsigned long long q = E.q0 + (st ? E.qo : 0u) + k;
	uint4 *vp = reinterpret_cast<uint4 *>(E.verts + 4 * q);
	vp[0] = make_uint4(v[0].x, v[0].y, v[1].x, v[1].y);
	vp[1] = make_uint4(v[2].x, v[2].y, v[3].x, v[3].y);
	const uint32_t m = k / kQuadsPerMesh, r = k - m * kQuadsPerMesh;
	// The reference reads the base index before closing a full mesh, so the first quad of every
	// continuation mesh indexes from 65,532 (BlockMeshAlgo.hpp:273-279, 397-403).
	const uint32_t b = (k > 0 && r == 0) ? 65532u : r * 4u;
	uint32_t *ip = reinterpret_cast<uint32_t *>(E.idx + 6 * q);
	if (flip) {
		ip[0] = b | ((b + 1) << 16);
		ip[1] = (b + 2) | (b << 16);
		ip[2] = (b + 2) | ((b + 3) << 16);
	} else {
		ip[0] = (b + 1) | ((b + 2) << 16);
		ip[1] = (b + 3) | (b << 16);
		ip[2] = (b + 1) | ((b + 3) << 16);
	}
	if (k > 0 && r == 0)
		S.trig[st][m - 1] = g;
}

// ------------------------------------------------------------------------------------- staging

// Stages the block classes of [-1, 32]^3, one warp per (y, z) row with lanes over x (twelve rows in
// flight), and the x-row bit planes of opaque full cubes and of blank blocks (from the chunk planes
// where there are planes, else built by ballots). Returns true when the chunk can produce no quad:
// every inner block has no texture and no custom mesh, or every inner block and every block of the
// six adjacent layers is an opaque full cube; has_custom: some inner block has a custom mesh.
// The staging scratch (the plane-mask memory): the chunk's 32 KB of class ids, the 132 apron rows
// (32 bytes each), then as many of the chunk's stored level planes (4 KB each) as fit.
constexpr int kStagedLevelOff = 32768 + 32 * (kCls * kCls - kChunk * kChunk);
constexpr int kStagedLevels = (int)((sizeof(Smem::u) - kStagedLevelOff) / (kPlaneWords * 4)) < 2 * kLevels
                                  ? (int)((sizeof(Smem::u) - kStagedLevelOff) / (kPlaneWords * 4))
                                  : 2 * kLevels;
static_assert(kStagedLevelOff % 16 == 0 && kStagedLevels >= 1 && kStagedLevels <= 16, "level copies fit the scratch");

__device__ bool stage_classes(Smem &S, const DevTables &T, bool &has_custom) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	constexpr int kRows = kCls * kCls, kBatch = 12; // 1156 rows; 12 in flight per warp
	constexpr int kApronRows = kRows - kChunk * kChunk; // 132
	const uint8_t *own = reinterpret_cast<const uint8_t *>(&S.u);
	if (S.pln[26]) {
		// The blank test first, from the layer summaries of the chunk and its six face neighbours
		// (one warp, 32 words each), so a blank chunk stages nothing.
		__shared__ uint32_t s_blank, s_custom, s_staged;
		if (warp == 0) {
			if (S.lvl[26]) { // the chunk's stored (non-uniform) level planes, the first kStagedLevels of them staged
				const uint32_t fl = lane < 2 * kLevels ? S.lfl[26][lane / kLevels] : 0u;
				const int t = lane % kLevels + 1;
				const bool stored = lane < 2 * kLevels && !level_empty(fl, t) && !level_full(fl, t);
				const uint32_t m = __ballot_sync(0xffffffffu, stored);
				const int slot = __popc(m & ((1u << lane) - 1u));
				const bool staged = stored && slot < kStagedLevels;
				if (lane < 2 * kLevels)
					S.lvl_slot[lane] = staged ? (int8_t)slot : (int8_t)-1;
				if (staged)
					S.lvl_plane[slot] = (int8_t)lane;
				if (lane == 0)
					s_staged = min(__popc(m), kStagedLevels);
			}
			const uint32_t mine = __ldg(S.pln[26] + kPlaneLayerOff + lane);
			const uint32_t xm = __ldg(S.pln[nb_index(-1, 0, 0)] + kPlaneLayerOff + lane);
			const uint32_t xp = __ldg(S.pln[nb_index(kChunk, 0, 0)] + kPlaneLayerOff + lane);
			const uint32_t zm = __ldg(S.pln[nb_index(0, 0, -1)] + kPlaneLayerOff + lane);
			const uint32_t zp = __ldg(S.pln[nb_index(0, 0, kChunk)] + kPlaneLayerOff + lane);
			const uint32_t ym = lane == 0 ? __ldg(S.pln[nb_index(0, -1, 0)] + kPlaneLayerOff + 31) : 0u;
			const uint32_t yp = lane == 0 ? __ldg(S.pln[nb_index(0, kChunk, 0)] + kPlaneLayerOff + 0) : 0u;
			const uint32_t open = (mine & kLayerOpen) | (xm & kLayerOpenX31) | (xp & kLayerOpenX0) |
			                      (zm & kLayerOpenZ31) | (zp & kLayerOpenZ0) | ((ym | yp) & kLayerOpen);
			const bool blank = !__any_sync(0xffffffffu, mine & kLayerContent) || !__any_sync(0xffffffffu, open);
			const bool custom = __any_sync(0xffffffffu, mine & kLayerCustom);
			if (lane == 0)
				s_blank = blank, s_custom = custom;
		}
		__syncthreads();
		has_custom = s_custom != 0;
		if (s_blank)
			return true;
		// The chunk's own 32 KB of class ids and the 132 x-rows of the apron (y or z outside [0, 32),
		// x in [0, 32), 32 bytes each from a neighbour's planes) are copied into the plane-mask
		// scratch (unused until the light and plane passes) by asynchronous 16-byte copies, all in
		// flight at once.
		const char *src = reinterpret_cast<const char *>(S.pln[26] + kPlaneClassOff);
		const uint32_t dst = (uint32_t)__cvta_generic_to_shared(own);
		for (int i = threadIdx.x; i < 32768 / 16; i += kThreads)
			asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16 * i), "l"(src + 16 * i) : "memory");
		for (int i = threadIdx.x; i < 2 * kApronRows; i += kThreads) {
			const int a = i >> 1, half = i & 1;
			const int y = a < 34 ? -1 : (a < 68 ? kChunk : (a - 68) >> 1);
			const int z = a < 34 ? a - 1 : (a < 68 ? a - 35 : (((a - 68) & 1) ? kChunk : -1));
			const char *row = reinterpret_cast<const char *>(S.pln[nb_index(0, y, z)] + kPlaneClassOff) +
			                  ((y & 31) * kChunk + (z & 31)) * kChunk + 16 * half;
			asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 32768 + 32 * a + 16 * half), "l"(row)
			             : "memory");
		}
		// With the batch light pass's level planes, up to kStagedLevels stored level planes of the
		// chunk itself (4 KB each) follow the apron rows, copied the same way.
		const bool lit = S.lvl[26] != nullptr;
		if (lit) {
			const uint32_t nw = s_staged * (kPlaneWords / 4);
			for (uint32_t i = threadIdx.x; i < nw; i += kThreads) {
				const uint32_t slot = i / (kPlaneWords / 4), q = i % (kPlaneWords / 4);
				const uint32_t *p = S.lvl[26] + (size_t)S.lvl_plane[slot] * kPlaneWords + 4 * q;
				asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + kStagedLevelOff + 16 * i), "l"(p)
				             : "memory");
			}
		}
		asm volatile("cp.async.commit_group;" ::: "memory");
		for (int i = threadIdx.x; i < 256; i += kThreads)
			S.classes[i] = T.classes[i];
		// With the batch light pass's level planes, the light of the apron rows and of the x-edge
		// pieces is decoded after the row bits below (its loads overlapping the copies still in
		// flight), that of the chunk's own rows after the copies, and each row is written together
		// with its class ids as whole cells; otherwise the class ids go in with light 0, for the
		// relight to raise.
		uint8_t *const hi = reinterpret_cast<uint8_t *>(S.cell) + 1;
		// First, one thread per row of [-1, 32]^2: the opaque-cube and blank bits of the row from
		// its chunk's planes with the x = -1 and x = 32 bits from the x neighbours' (bit x + 1), and
		// the class ids of the row's two edge cells.
		for (int row = threadIdx.x; row < kRows; row += kThreads) {
			const int y = row / kCls - 1, z = row % kCls - 1, ry = ((y & 31) << 5) | (z & 31);
			const uint32_t *P = S.pln[nb_index(0, y, z)], *Pm = S.pln[nb_index(-1, y, z)], *Pp = S.pln[nb_index(kChunk, y, z)];
			const uint32_t oc = __ldg(P + kPlaneOpaque * kPlaneWords + ry), em = __ldg(P + kPlaneEmpty * kPlaneWords + ry);
			const uint32_t ocm = __ldg(Pm + kPlaneOpaque * kPlaneWords + ry), emm = __ldg(Pm + kPlaneEmpty * kPlaneWords + ry);
			const uint32_t ocp = __ldg(Pp + kPlaneOpaque * kPlaneWords + ry), emp = __ldg(Pp + kPlaneEmpty * kPlaneWords + ry);
			const uint8_t e0 = class_byte(S, -1, y, z), e1 = class_byte(S, kChunk, y, z);
			S.aux.pl.oc[row] = (uint64_t)(ocm >> 31) | ((uint64_t)oc << 1) | ((uint64_t)(ocp & 1u) << 33);
			S.aux.pl.em[row] = (uint64_t)(emm >> 31) | ((uint64_t)em << 1) | ((uint64_t)(emp & 1u) << 33);
			if (lit) {
				hi[2 * (row * kCls)] = e0;
				hi[2 * (row * kCls + kCls - 1)] = e1;
			} else {
				S.cell[row * kCls] = (uint16_t)(e0 << 8);
				S.cell[row * kCls + kCls - 1] = (uint16_t)(e1 << 8);
			}
		}
		// the light of apron row a (thread a < 132) or edge piece threadIdx.x - 132 is decoded now and
		// the apron row's kept in registers until its class ids have arrived; edge pieces are written now
		constexpr int kOtherItems = kApronRows + 2 * kLt * 3;
		static_assert(kOtherItems <= kThreads && kChunk * kChunk == kThreads, "one item of each kind per thread");
		uint64_t lrow[4];
		int arow = -1;
		if (lit && threadIdx.x < kOtherItems) {
			int it = kLt * kLt + (threadIdx.x - kApronRows);
			if (threadIdx.x < kApronRows) {
				const int a = threadIdx.x;
				const int y = a < 34 ? -1 : (a < 68 ? kChunk : (a - 68) >> 1);
				const int z = a < 34 ? a - 1 : (a < 68 ? a - 35 : (((a - 68) & 1) ? kChunk : -1));
				it = arow = (y + 1) * kCls + (z + 1);
			}
			light_item(S, it, lrow);
		}
		asm volatile("cp.async.wait_group 0;" ::: "memory");
		__syncthreads();
		if (lit) { // light and class id of the cells x in [0, 32) of each row, as whole cells
			if (arow >= 0)
				write_row_cells(S, arow, lrow, own + 32768 + 32 * threadIdx.x);
			const int y = threadIdx.x >> 5, z = threadIdx.x & 31; // the chunk's own row of this thread
			light_own_row(S, y, z, reinterpret_cast<const uint32_t *>(own + kStagedLevelOff), lrow);
			write_row_cells(S, (y + 1) * kCls + z + 1, lrow, own + (y * kChunk + z) * kChunk);
			__syncthreads();
			return false;
		}
		// without light-pass levels: class ids of the cells x in [0, 32) of every row, from the copies
		// (light 0 for the relight to raise); one warp per row, lanes over x
		for (int row0 = warp * kBatch; row0 < kRows; row0 += kWarps * kBatch) {
			uint8_t c[kBatch];
#pragma unroll
			for (int j = 0; j < kBatch; ++j) {
				const int row = min(row0 + j, kRows - 1), y = row / kCls - 1, z = row % kCls - 1;
				const bool inner = (unsigned)y < (unsigned)kChunk && (unsigned)z < (unsigned)kChunk;
				const int a = y < 0 ? z + 1 : (y >= kChunk ? 35 + z : 68 + 2 * y + (z >= kChunk)); // apron row
				c[j] = own[inner ? lane + (y * kChunk + z) * kChunk : 32768 + 32 * a + lane];
			}
#pragma unroll
			for (int j = 0; j < kBatch; ++j) {
				if (row0 + j >= kRows) // the same for the whole warp
					break;
				S.cell[(row0 + j) * kCls + lane + 1] = (uint16_t)(c[j] << 8);
			}
		}
		__syncthreads();
		return false;
	}
	for (int i = threadIdx.x; i < 256; i += kThreads) {
		const DevClass k = T.classes[i];
		S.classes[i] = k;
		S.cflags[i] = k.flags;
		// classes with a custom mesh, as a 256-bit set
		const uint32_t cm = __ballot_sync(0xffffffffu, (k.mesh_meta & 3u) != 0);
		if ((threadIdx.x & 31) == 0)
			S.cmesh[i >> 5] = cm;
	}
	__syncthreads();
	bool content = false, open = false, custom = false;
	{
		for (int row0 = warp * kBatch; row0 < kRows; row0 += kWarps * kBatch) {
			uint8_t c[kBatch], ce[kBatch];
			uint16_t raw[kBatch], rawe[kBatch];
#pragma unroll
			for (int j = 0; j < kBatch; ++j) {
				const int row = min(row0 + j, kRows - 1), y = row / kCls - 1, z = row % kCls - 1;
				raw[j] = raw_at(S, lane, y, z);
				rawe[j] = lane < 2 ? raw_at(S, lane ? kChunk : -1, y, z) : (uint16_t)0;
			}
#pragma unroll
			for (int j = 0; j < kBatch; ++j) {
				c[j] = __ldg(T.class_of + raw[j]);
				ce[j] = __ldg(T.class_of + rawe[j]);
			}
#pragma unroll
			for (int j = 0; j < kBatch; ++j) {
				const int row = row0 + j, y = row / kCls - 1, z = row % kCls - 1;
				if (row >= kRows) // the same for the whole warp
					break;
				uint16_t *dst = S.cell + row * kCls;
				dst[lane + 1] = (uint16_t)(c[j] << 8);
				if (lane < 2)
					dst[lane ? kCls - 1 : 0] = (uint16_t)(ce[j] << 8);
				const uint8_t f = S.cflags[c[j]], fe = S.cflags[ce[j]];
				const uint32_t oc = __ballot_sync(0xffffffffu, f & kFOpaqueCube);
				const uint32_t em = __ballot_sync(0xffffffffu, f & kFEmpty);
				const uint32_t oce = __ballot_sync(0xffffffffu, lane < 2 && (fe & kFOpaqueCube));
				const uint32_t eme = __ballot_sync(0xffffffffu, lane < 2 && (fe & kFEmpty));
				if (lane == 0) {
					S.aux.pl.oc[row] = (uint64_t)(oce & 1u) | ((uint64_t)oc << 1) | ((uint64_t)((oce >> 1) & 1u) << 33);
					S.aux.pl.em[row] = (uint64_t)(eme & 1u) | ((uint64_t)em << 1) | ((uint64_t)((eme >> 1) & 1u) << 33);
				}
				const bool yin = y >= 0 && y < kChunk, zin = z >= 0 && z < kChunk;
				if (yin && zin) {
					content |= !(f & kFEmpty);
					open |= !(f & kFOpaqueCube) || (lane < 2 && !(fe & kFOpaqueCube));
					custom |= (S.cmesh[c[j] >> 5] >> (c[j] & 31)) & 1u;
				} else if (yin || zin) { // a face-adjacent layer row (x in [0, 32))
					open |= !(f & kFOpaqueCube);
				}
			}
		}
	}
	content = __syncthreads_or(content);
	open = __syncthreads_or(open);
	has_custom = __syncthreads_or(custom);
	return !content || !open;
}

// ------------------------------------------------------------------------------- custom meshes

// Faces of the custom mesh of inner block (x, y, z); returns the count, fills `faces` if given.
__device__ uint32_t custom_faces(const Smem &S, int x, int y, int z, hc_mesh_face *faces) {
	const DevClass &k = S.classes[class_at(S, x, y, z)];
	const uint32_t kind = k.mesh_meta & 3u;
	if (kind == HC_MESH_STATIC) {
		const uint32_t n = k.mesh_meta >> 2;
		if (faces)
			for (uint32_t i = 0; i < n; ++i)
				faces[i] = c_static_faces[k.mesh_first + i];
		return n;
	}
	if (kind == HC_MESH_FLOW) {
		uint16_t t6[6];
		uint32_t n;
		flow_mesh_at(S, x, y, z, (uint8_t)(k.mesh_meta >> 2), faces, &n, t6);
		return n;
	}
	return 0;
}

// Stream counts of the custom faces of inner blocks [first, first + kBlocksPerThread).
__device__ void custom_count(const Smem &S, int first, uint32_t &co, uint32_t &ct) {
	co = ct = 0;
	for (int i = first; i < first + kBlocksPerThread; ++i) {
		const int x = i & 31, z = (i >> 5) & 31, y = i >> 10;
		const DevClass &k = S.classes[class_at(S, x, y, z)];
		const uint32_t kind = k.mesh_meta & 3u;
		if (kind == HC_MESH_STATIC) {
			for (uint32_t f = 0; f < (uint32_t)(k.mesh_meta >> 2); ++f) {
				if (tex_transpass(c_static_faces[k.mesh_first + f].texture))
					++ct;
				else
					++co;
			}
		} else if (kind == HC_MESH_FLOW) {
			ct += custom_faces(S, x, y, z, nullptr); // liquid faces use the transparent pass
		}
	}
}

// Trilinear light of a custom-mesh vertex (BlockMeshAlgo.hpp:165-196).
__device__ __forceinline__ uint32_t lerp16(uint32_t a, uint32_t b, uint32_t t) { return a * (16u - t) + b * t; }
__device__ __forceinline__ uint32_t ceil4096(uint32_t a) { return (a >> 12) + ((a & 4095u) ? 1u : 0u); }
__device__ __forceinline__ uint32_t tri(uint32_t l0, uint32_t l1, uint32_t l2, uint32_t l3, uint32_t h0, uint32_t h1,
                                        uint32_t h2, uint32_t h3, uint32_t du, uint32_t dv, uint32_t dw) {
	return ceil4096(lerp16(lerp16(lerp16(l0, l1, du), lerp16(l3, l2, du), dv),
	                       lerp16(lerp16(h0, h1, du), lerp16(h3, h2, du), dv), dw));
}

__device__ void custom_emit(Smem &S, const Emit &E, int first, uint32_t ko, uint32_t kt, uint32_t g) {
	for (int i = first; i < first + kBlocksPerThread; ++i) {
		const int x = i & 31, z = (i >> 5) & 31, y = i >> 10;
		const DevClass &kc = S.classes[class_at(S, x, y, z)];
		if ((kc.mesh_meta & 3u) == HC_MESH_NONE)
			continue;
		hc_mesh_face faces[HC_MAX_MESH_FACES];
		const uint32_t n = custom_faces(S, x, y, z, faces);
		const uint32_t base[3] = {(uint32_t)x << 4, (uint32_t)y << 4, (uint32_t)z << 4};
		int cur_face = 255, cur_axis = 0, ua = 0, va = 0;
		Light4 lo{0, 0, 0}, hi{0, 0, 0};
		for (uint32_t f = 0; f < n; ++f) {
			const hc_mesh_face &mf = faces[f];
			if (mf.light_face != cur_face) {
				cur_face = mf.light_face;
				cur_axis = cur_face >> 1;
				ua = (cur_axis + 1) % 3;
				va = (cur_axis + 2) % 3;
				if (cur_face & 1) {
					const int t = ua;
					ua = va, va = t;
				}
				int op[3] = {x, y, z}, ne[3] = {x, y, z};
				const int d = 1 - ((cur_face & 1) << 1);
				op[cur_axis] -= d;
				ne[cur_axis] += d;
				lo = light4(S, cur_face, op[0], op[1], op[2]);
				if (id_indirect(class_at(S, ne[0], ne[1], ne[2])))
					hi = light4(S, cur_face, x, y, z);
				else
					hi = lo;
			}
			const int st = tex_transpass(mf.texture) ? 1 : 0;
			uint2 v[4];
			uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0, 0, 0};
			for (int c = 0; c < 4; ++c) {
				const hc_mesh_vertex &mv = mf.v[c];
				const uint32_t p[3] = {base[0] + mv.pos[0], base[1] + mv.pos[1], base[2] + mv.pos[2]};
				for (int a = 0; a < 3; ++a) {
					mn[a] = min(mn[a], p[a]);
					mx[a] = max(mx[a], p[a]);
				}
				const uint32_t du = mv.pos[ua], dv = mv.pos[va];
				uint32_t dw = mv.pos[cur_axis] < 16 ? mv.pos[cur_axis] : 16u;
				if (cur_face & 1)
					dw = 16u - dw;
				uint32_t ao = mv.ao;
				if (ao == 4)
					ao = tri(ao_get(lo.ao, 0), ao_get(lo.ao, 1), ao_get(lo.ao, 2), ao_get(lo.ao, 3), ao_get(hi.ao, 0),
					         ao_get(hi.ao, 1), ao_get(hi.ao, 2), ao_get(hi.ao, 3), du, dv, dw);
				const uint32_t sun = tri(l4_get(lo.sun, 0), l4_get(lo.sun, 1), l4_get(lo.sun, 2), l4_get(lo.sun, 3),
				                         l4_get(hi.sun, 0), l4_get(hi.sun, 1), l4_get(hi.sun, 2), l4_get(hi.sun, 3), du, dv, dw);
				const uint32_t torch =
				    tri(l4_get(lo.torch, 0), l4_get(lo.torch, 1), l4_get(lo.torch, 2), l4_get(lo.torch, 3),
				        l4_get(hi.torch, 0), l4_get(hi.torch, 1), l4_get(hi.torch, 2), l4_get(hi.torch, 3), du, dv, dw);
				v[c] = pack_vertex(p[0], p[1], p[2], mf.axis, mf.render_face, ao & 0xffu, sun & 0xffu, torch & 0xffu,
				                   mf.texture);
			}
			const uint32_t kq = st ? kt : ko;
			put_quad(S, E, st, kq, g, v, true);
			aabb_add(S, st, kq / kQuadsPerMesh, mn, mx);
			if (st)
				++kt;
			else
				++ko;
			++g;
		}
	}
}

// -------------------------------------------------------------------------------- face planes

__device__ __forceinline__ int plane_id(int axis, int slice, int inv) { return axis * 66 + slice * 2 + inv; }

// 32 x 32 bit transpose across a warp: lane r holds row r (bit c = column c) on entry and column r
// (bit c = row c) on return. Five butterfly rounds swap ever smaller off-diagonal blocks.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
	const int lane = threadIdx.x & 31;
	uint32_t m = 0x0000ffffu;
#pragma unroll
	for (int j = 16; j != 0; j >>= 1, m ^= m << j) {
		const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
		const bool upper = (lane & j) != 0;
		const uint32_t t = (((upper ? y : x) >> j) ^ (upper ? x : y)) & m;
		x ^= upper ? t : (t << j);
	}
	return x;
}

// Pass 1 (before the relight): visibility of both face planes of every slice from the opaque-cube
// and blank planes. Between an opaque cube and a blank block only the cube's face shows; two cubes
// or two blanks show nothing (BlockTexture::Show); any pair involving another block ("complex":
// transparent, liquid, custom mesh) is left to pass 1b. Writes visible bits to masks[.][u][0],
// complex candidates to [.][u][1], zero transparent-pass bits to [.][u][3]. Lane = plane row.
__device__ void plane_visibility(Smem &S) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	constexpr uint64_t k34 = (1ull << 34) - 1ull;
	// y and z slices: rows straight from the x-row planes (bit x + 1 -> plane bit x)
	for (int sl = warp; sl < 66; sl += kWarps) {
		const int a = 1 + sl / 33, s = sl % 33, u = lane;
		// cells n (slice coordinate s - 1) and p (slice coordinate s) of plane row u
		const int rn = a == 1 ? (u + 1) + kCls * s : s + kCls * (u + 1);
		const int rp = a == 1 ? (u + 1) + kCls * (s + 1) : (s + 1) + kCls * (u + 1);
		const uint64_t ocn = S.aux.pl.oc[rn], emn = S.aux.pl.em[rn], ocp = S.aux.pl.oc[rp], emp = S.aux.pl.em[rp];
		const uint32_t cx = (uint32_t)((((~(ocn | emn)) | (~(ocp | emp))) & k34) >> 1);
		const uint32_t va = s != 0 ? (uint32_t)((ocn & emp) >> 1) : 0u;
		const uint32_t vb = s != 32 ? (uint32_t)((ocp & emn) >> 1) : 0u;
		uint32_t *mA = S.u.masks[plane_id(a, s, 0)][u];
		uint32_t *mB = S.u.masks[plane_id(a, s, 1)][u];
		mA[0] = va, mA[1] = s != 0 ? cx : 0u, mA[3] = 0;
		mB[0] = vb, mB[1] = s != 32 ? cx : 0u, mB[3] = 0;
	}
	// x slices: per row y, lane = z holds the x-row words with the faces of every slice (bit s);
	// a warp bit transpose turns slices 0-31 into plane rows over z (lane = slice), a ballot slice
	// 32. Row words are written whole: the equal-below word is cleared again by the key pass.
	for (int y = warp; y < kChunk; y += kWarps) {
		const int r = (lane + 1) + kCls * (y + 1);
		const uint64_t oc = S.aux.pl.oc[r], em = S.aux.pl.em[r];
		const uint64_t fa = oc & (em >> 1), fb = (oc >> 1) & em; // bit s: face at slice s
		const uint64_t c = ~(oc | em) & k34, cxp = c | (c >> 1);
		const uint32_t va = warp_transpose32((uint32_t)fa), vb = warp_transpose32((uint32_t)fb);
		const uint32_t cx = warp_transpose32((uint32_t)cxp);
		const uint32_t va32 = __ballot_sync(0xffffffffu, (fa >> 32) & 1u);
		const uint32_t cx32 = __ballot_sync(0xffffffffu, (cxp >> 32) & 1u);
		const int sl = lane; // slices 0-31: face B always, face A from slice 1
		*reinterpret_cast<uint4 *>(S.u.masks[plane_id(0, sl, 0)][y]) =
		    sl != 0 ? make_uint4(va, cx, 0u, 0u) : make_uint4(0u, 0u, 0u, 0u);
		*reinterpret_cast<uint4 *>(S.u.masks[plane_id(0, sl, 1)][y]) = make_uint4(vb, cx, 0u, 0u);
		if (lane == 0) { // slice 32: face A only
			*reinterpret_cast<uint4 *>(S.u.masks[plane_id(0, 32, 0)][y]) = make_uint4(va32, cx32, 0u, 0u);
			*reinterpret_cast<uint4 *>(S.u.masks[plane_id(0, 32, 1)][y]) = make_uint4(0u, 0u, 0u, 0u);
		}
	}
}

// Pass 1b: exact Show for the complex candidates of one plane's rows (texture lookups, dynamic
// liquid textures), and transparent-pass bits of the faces it shows. Lane = plane row. Run by the
// warp that takes the plane (or half of it) for its keys: rows [lo, r1) are resolved and returned
// as visible bits (0 for other rows); rows [r0, r1) are written back. Row lo < r0 is the row above
// a second half, read from its copy `side` (its words in the masks belong to the other half).
__device__ __forceinline__ uint32_t plane_complex_one(Smem &S, int p, int lo = 0, int r0 = 0, int r1 = 32,
                                                      const uint32_t *side = nullptr) {
	const int lane = threadIdx.x & 31;
	uint32_t *m = S.u.masks[p][lane];
	const bool in = lane >= lo && lane < r1, ctx = lane < r0;
	uint32_t vis = in ? (ctx ? side[0] : m[0]) : 0u;
	uint32_t cx = in ? (ctx ? side[1] : m[1]) : 0u;
	if (!__any_sync(0xffffffffu, cx != 0))
		return vis;
	const int a = p / 66, s = (p % 66) >> 1, inv = p & 1;
	uint32_t tp = 0;
	while (cx) {
		const int v = __ffs(cx) - 1;
		cx &= cx - 1;
		int x, y, z;
		to_xyz(a, s, lane, v, x, y, z);
		int nx = x, ny = y, nz = z;
		(a == 0 ? nx : (a == 1 ? ny : nz)) -= 1;
		const uint16_t ta = get_tex(S, nx, ny, nz, 2 * a), tb = get_tex(S, x, y, z, 2 * a + 1);
		const uint16_t mine = inv ? tb : ta, other = inv ? ta : tb;
		if (show(mine, other)) {
			vis |= 1u << v;
			if (tex_transpass(mine))
				tp |= 1u << v;
		} else {
			vis &= ~(1u << v);
		}
	}
	if (in && !ctx) {
		m[0] = vis;
		m[3] = tp;
	}
	__syncwarp();
	return vis;
}

// Position of the n-th (0-based) set bit of mask (n < popc(mask)), by halving the search window.
__device__ __forceinline__ int nth_set_bit(uint32_t mask, uint32_t n) {
	int pos = 0;
#pragma unroll
	for (int w = 16; w > 0; w >>= 1) {
		const uint32_t low = mask & ((1u << w) - 1u);
		const uint32_t c = __popc(low);
		if (n >= c) {
			n -= c;
			mask >>= w;
			pos += w;
		} else {
			mask = low;
		}
	}
	return pos;
}

struct Key {
	uint32_t tex_ao, sun, torch;
};
__device__ __forceinline__ bool key_eq(const Key &a, const Key &b) {
	return a.tex_ao == b.tex_ao && a.sun == b.sun && a.torch == b.torch;
}
__device__ __forceinline__ Key shfl_down_key(const Key &k) {
	return Key{__shfl_down_sync(0xffffffffu, k.tex_ao, 1), __shfl_down_sync(0xffffffffu, k.sun, 1),
	           __shfl_down_sync(0xffffffffu, k.torch, 1)};
}

// Key of the face of plane (a, s, inv) at cell (u, v): texture, AO and the smoothed light.
__device__ __forceinline__ Key face_key(const Smem &S, int a, int s, int inv, int u, int v, uint16_t *tex_out, Light4 *l_out) {
	int x, y, z;
	to_xyz(a, s, u, v, x, y, z);
	if (!inv)
		(a == 0 ? x : (a == 1 ? y : z)) -= 1;
	const uint16_t t = get_tex(S, x, y, z, 2 * a + inv);
	const Light4 l = light4(S, 2 * a + inv, x, y, z);
	if (tex_out)
		*tex_out = t;
	if (l_out)
		*l_out = l;
	return Key{(uint32_t)t | (l.ao << 16), l.sun, l.torch};
}

__device__ void plane_count_one(Smem &S, int p);

// Warp exclusive prefix sum over lanes of a value packing two 16-bit counts; *total gets the sum.
__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t x, uint32_t *total) {
	const int lane = threadIdx.x & 31;
	uint32_t incl = x;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
		if (lane >= d)
			incl += o;
	}
	*total = __shfl_sync(0xffffffffu, incl, 31);
	return incl - x;
}

// Heavy face planes (see split_heavy_planes; the kMaxSplit heaviest at most) are keyed in row parts by
// several warps (one part per kPartWeight of weight, two to kMaxParts), so that a heavy plane does not hold the
// key phase open; the warp that finishes last merges and counts the plane. The split rows balance
// the weights (visible faces and complex candidates) of the parts. The row above each part after the
// first is keyed by that part too (for the equal-below bits of that row): it reads the row's visible
// and complex words from a copy taken here, as the part before rewrites them.
constexpr uint32_t kSplitMin = 128;
constexpr uint32_t kPartWeight = 96; // a split plane gets one part per this much weight (2 to kMaxParts)

// After order_planes (plane weights in seg_base). Returns how many planes are split (every thread).
__device__ int split_heavy_planes(Smem &S, int live) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t *weight = &S.seg_base[0][0];
	// A plane is split when it is heavy against the chunk's whole key work: weight >= kSplitMin and
	// at least twice a warp's even share (on a chunk of many heavy planes the warps are kept busy by
	// whole planes, and parts would only add context rows and merges). The split planes are the
	// longest prefix of the order (at most kMaxSplit) whose weights pass, so split plane k is order[k].
	__shared__ int s_nsplit;
	if (warp == 0) {
		uint32_t sum = 0;
		for (int q = lane; q < live; q += 32)
			sum += weight[S.order[q]];
		sum = __reduce_add_sync(0xffffffffu, sum);
		if (lane == 0) {
			const uint32_t min_split = max(kSplitMin, 2 * sum / kWarps);
			int k = 0;
			while (k < kMaxSplit && k < live && weight[S.order[k]] >= min_split)
				++k;
			s_nsplit = k;
		}
	}
	__syncthreads();
	const int nsplit = s_nsplit;
	if (warp < nsplit) {
		const int p = S.order[warp];
		const uint32_t w = __popc(S.u.masks[p][lane][0] | S.u.masks[p][lane][1]);
		uint32_t tot;
		const uint32_t ex = warp_excl_scan(w, &tot);
		const int parts = (int)min((uint32_t)kMaxParts, max(2u, (tot + kPartWeight - 1) / kPartWeight));
		int prev = 0;
		for (int q = 1; q < parts; ++q) { // part q starts at the row where the weight passes q / parts
			int r = __ffs(__ballot_sync(0xffffffffu, (ex + w) * (uint32_t)parts > (uint32_t)q * tot)) - 1;
			r = min(max(r, prev + 1), 32 - (parts - q));
			if (lane == 0) {
				S.split_rows[warp][q] = (uint8_t)r;
				S.split_side[warp][q][0] = S.u.masks[p][r - 1][0];
				S.split_side[warp][q][1] = S.u.masks[p][r - 1][1];
			}
			prev = r;
		}
		if (lane == 0) {
			S.split_rows[warp][0] = 0;
			S.split_rows[warp][parts] = 32;
			S.split_first[warp + 1] = (uint8_t)parts; // a count here; turned into offsets below
			S.split_done[warp] = 0;
		}
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		S.split_first[0] = 0;
		for (int k = 0; k < nsplit; ++k)
			S.split_first[k + 1] = (uint8_t)(S.split_first[k] + S.split_first[k + 1]);
	}
	__syncthreads();
	return nsplit;
}

// Next key-pass item for the calling warp: plane | part << 8 | split index << 12, part 0 = the whole
// plane, q + 1 = part q of split plane k. The parts of the split planes come first, then the other
// planes heaviest first. A whole plane is recorded as this CTA's when taken, a split one by the
// warp that merges it.
__device__ __forceinline__ int claim_item(Smem &S, const Split &sp, int live, int nsplit) {
	if (sp.c > 1)
		return claim_plane(S, sp, live);
	int r = kPlanes;
	if ((threadIdx.x & 31) == 0) {
		const int j = (int)atomicAdd(&S.misc[kClaimKeys], 1u);
		const int nparts = S.split_first[nsplit];
		if (j < nparts) {
			int k = 0;
			while (j >= S.split_first[k + 1])
				++k;
			r = (int)S.order[k] | ((1 + j - S.split_first[k]) << 8) | (k << 12);
		} else {
			const int jj = j - nparts + nsplit;
			r = jj < live ? (int)S.order[jj] : kPlanes;
			if (r < kPlanes)
				S.mine[atomicAdd(&S.misc[kMine], 1u)] = (uint8_t)r;
		}
	}
	return __shfl_sync(0xffffffffu, r, 0);
}

__device__ void plane_count_one(Smem &S, int p);

// Keyed faces of a plane's rows (lane = row): the visible words V with the lone faces left out.
// A lone face (no visible face left, right, above or below it in the plane) takes part in no
// equality: it is a quad of its own whatever its key, so it is not keyed (the emission computes its
// light). Rows next to a row the calling warp does not resolve (the other half of a split plane,
// outside [lo, r1)) are keyed whole. Every visible neighbour of a keyed face is keyed too.
__device__ __forceinline__ uint32_t keyed_faces(uint32_t V, int lo, int r1) {
	const int lane = threadIdx.x & 31;
	const uint32_t Vu1 = __shfl_up_sync(0xffffffffu, V, 1), Vd1 = __shfl_down_sync(0xffffffffu, V, 1);
	const uint32_t Vup = lane == 0 ? 0u : Vu1, Vdn = lane == 31 ? 0u : Vd1;
	const bool resolved_around = !(lane == r1 - 1 && r1 < 32) && !(lane == lo && lo > 0);
	const uint32_t lone = resolved_around ? (V & ~(V << 1) & ~(V >> 1) & ~Vup & ~Vdn) : 0u;
	return V & ~lone;
}

// Inclusive warp scan (lane = row) of a row count.
__device__ __forceinline__ uint32_t row_scan(uint32_t cnt) {
	const int lane = threadIdx.x & 31;
	uint32_t incl = cnt;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
		if (lane >= d)
			incl += o;
	}
	return incl;
}

// Pass 2 (after the relight): equal-to-right and equal-to-below masks of every plane, each plane
// then merged and counted by the warp that built its masks (no block barrier in between). The visible
// faces of a plane are taken in batches of whole rows (at most 32 faces), one face per lane, so
// the light keys are computed by full warps; a face's right neighbour is the next lane and its
// upper neighbour sits in this batch or in the previous one. A half plane keys rows [lo, r1) and
// writes the equal-right bits of rows [r0, r1) and the equal-below bits of rows [lo, r1 - 1).
__device__ void plane_keys(Smem &S, const Split &sp, int live, int nsplit) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int item = claim_item(S, sp, live, nsplit); (item & 255) < kPlanes; item = claim_item(S, sp, live, nsplit)) {
		const int p = item & 255, part = (item >> 8) & 15, ks = item >> 12;
		const int r0 = part ? (int)S.split_rows[ks][part - 1] : 0, r1 = part ? (int)S.split_rows[ks][part] : 32;
		const int lo = r0 > 0 ? r0 - 1 : 0;
		const uint32_t V = plane_complex_one(S, p, lo, r0, r1, part > 1 ? S.split_side[ks][part - 1] : nullptr);
		uint32_t *mrow = S.u.masks[p][lane];
		if (lane >= r0 && lane < r1)
			mrow[1] = 0;
		if (lane >= lo && (lane < r1 - 1 || (lane == 31 && r1 == 32)))
			mrow[2] = 0;
		const bool any_face = __any_sync(0xffffffffu, V != 0);
		const uint32_t N = keyed_faces(V, lo, r1);
		const uint32_t cnt = __popc(N);
		const uint32_t incl = row_scan(cnt);
		const uint32_t start = incl - cnt;
		const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
		__syncwarp();
		const int a = p / 66, s = (p % 66) >> 1, inv = p & 1;
		Key prev{0, 0, 0};
		uint32_t prev_b = 0, b = 0;
		int ub = 0;
		while (b < total) {
			// rows [ub, ue) whose faces fit in 32 lanes from index b
			const uint32_t over = __ballot_sync(0xffffffffu, lane >= ub && incl > b + 32);
			const int ue = over ? __ffs(over) - 1 : 32;
			const uint32_t be = __shfl_sync(0xffffffffu, start, ue & 31);
			const uint32_t bend = ue < 32 ? be : total;
			// this lane's face: compacted index f = b + lane. The batch starts at row ub's first face
			// and every row holds at most 32 faces, so the rows of the batch that hold faces start
			// at distinct lanes: lane j's row is the one that starts at the last start at or below j.
			const uint32_t f = b + lane;
			const bool has = f < bend;
			const bool rin = lane >= ub && lane < ue && cnt > 0;
			const uint32_t M = __reduce_or_sync(0xffffffffu, rin ? 1u << (start - b) : 0u);
			const uint32_t upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
			if (rin) // each row of the batch records itself where its faces start
				S.row_of[warp][start - b] = (uint8_t)lane;
			__syncwarp();
			const int u = has ? S.row_of[warp][31 - __clz(M & upto)] : 0;
			__syncwarp();
			const uint32_t su = __shfl_sync(0xffffffffu, start, u); // every lane takes part
			const uint32_t k = has ? f - su : 0u;
			const uint32_t Nu = __shfl_sync(0xffffffffu, N, u);
			const int v = has ? nth_set_bit(Nu, k) : 0;
			Key key{0, 0, 0};
			if (has)
				key = face_key(S, a, s, inv, u, v, nullptr, nullptr);
			// right neighbour: next lane when (u, v + 1) is visible
			const Key right = shfl_down_key(key);
			const bool rv = has && v < 31 && ((Nu >> (v + 1)) & 1u);
			if (rv && u >= r0 && key_eq(key, right))
				atomicOr(&S.u.masks[p][u][1], 1u << v);
			// upper neighbour (u - 1, v)
			const uint32_t Nup = __shfl_sync(0xffffffffu, N, (u + 31) & 31);
			const uint32_t sup = __shfl_sync(0xffffffffu, start, (u + 31) & 31);
			const bool uv = has && u > lo && ((Nup >> v) & 1u);
			const uint32_t fi = sup + __popc(Nup & ((1u << v) - 1u));
			const int src_cur = (int)(fi - b) & 31, src_prev = (int)(fi - prev_b) & 31;
			const Key kc{__shfl_sync(0xffffffffu, key.tex_ao, src_cur), __shfl_sync(0xffffffffu, key.sun, src_cur),
			             __shfl_sync(0xffffffffu, key.torch, src_cur)};
			const Key kp{__shfl_sync(0xffffffffu, prev.tex_ao, src_prev), __shfl_sync(0xffffffffu, prev.sun, src_prev),
			             __shfl_sync(0xffffffffu, prev.torch, src_prev)};
			if (uv && key_eq(key, fi >= b ? kc : kp))
				atomicOr(&S.u.masks[p][u - 1][2], 1u << v);
			prev = key;
			prev_b = b;
			b = bend;
			ub = ue;
		}
		__syncwarp();
		if (part == 0) {
			if (any_face)
				plane_count_one(S, p);
			continue;
		}
		// a part: the warp that finishes last merges the plane (its masks are complete then)
		__threadfence_block();
		uint32_t done_before = 0;
		if (lane == 0)
			done_before = atomicAdd(&S.split_done[ks], 1u);
		if (__shfl_sync(0xffffffffu, done_before, 0) + 1u == (uint32_t)(S.split_first[ks + 1] - S.split_first[ks])) {
			__threadfence_block();
			if (lane == 0)
				S.mine[atomicAdd(&S.misc[kMine], 1u)] = (uint8_t)p;
			plane_count_one(S, p);
		}
	}
}

// Exact greedy scan of one plane from its masks (BlockMeshAlgo.hpp:345-477), one warp per plane.
// For each row u (in order) the quads starting in row u are its runs: maximal stretches of live
// (visible, not yet covered) cells whose right neighbours are equal (width first); every run then
// grows down over whole rows while each of its cells equals the one above (height). A run's height
// is therefore 1 + the least, over its columns, of the number of consecutive equal-below bits from
// row u down: lane v holds column v of the equal-below mask (transposed once per plane) and of the
// covered cells, and a segmented minimum over the run's lanes gives the height without walking the
// rows. Cells below row u can only be covered by quads of row u itself (a quad from a row above
// that reaches them also covers row u there), so runs never meet covered cells below.
// For every row with quads the whole warp calls t = on_starts(starts) as soon as the row's quad
// starts are known (so that what it starts, e.g. an atomic, overlaps the height search) and then
// on_row(t, u, starts, tmask, is_start, w, h); the quad of lane v (is_start) is (u, v, w, h) and its
// stream is bit v of tmask. Only the rows in `only` are scanned: a caller may leave out rows that
// no quad of another row reaches and whose own quads do not grow down (see plane_count_one).
template <typename G, typename F>
__device__ __forceinline__ void warp_merge_plane(const uint32_t (*m)[4], G &&on_starts, F &&on_row,
                                                 uint32_t only = 0xffffffffu) {
	const int lane = threadIdx.x & 31;
	const uint32_t rN = m[lane][0];
	uint32_t rows = __ballot_sync(0xffffffffu, rN != 0) & only;
	if (!rows)
		return;
	const uint32_t rE = m[lane][1], rT = m[lane][3];
	const uint32_t Dc = warp_transpose32(m[lane][2]); // bit r: cell (r, lane) equals cell (r + 1, lane)
	const uint32_t upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
	uint32_t Cc = 0;                                   // bit r: cell (r, lane) is covered
	while (rows) {
		const int u = __ffs(rows) - 1;
		rows &= rows - 1;
		const uint32_t live = __shfl_sync(0xffffffffu, rN, u) & ~__ballot_sync(0xffffffffu, (Cc >> u) & 1u);
		if (!live)
			continue;
		const uint32_t Eu = __shfl_sync(0xffffffffu, rE, u), Tu = __shfl_sync(0xffffffffu, rT, u);
		const uint32_t cont = live & (live << 1) & (Eu << 1); // bit v continues the run of v-1
		const uint32_t starts = live & ~cont;
		const uint32_t token = on_starts(starts);
		const bool in_run = (live >> lane) & 1u, is_start = (starts >> lane) & 1u;
		const uint32_t after = lane == 31 ? 0u : (cont >> (lane + 1));
		const int rem = __ffs(~after); // lanes from this one to the end of its run
		// rows below u this column can grow over, then the minimum over the rest of the run (all
		// heights are 1 when no cell of the row's runs equals the one below it)
		int h = 1;
		if (__any_sync(0xffffffffu, in_run && ((Dc >> u) & 1u))) {
			int dl = in_run ? __ffs(~(Dc >> u)) - 1 : 32;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				const int o = __shfl_down_sync(0xffffffffu, dl, d);
				if (d < rem)
					dl = min(dl, o);
			}
			h = __shfl_sync(0xffffffffu, dl, 31 - __clz(starts & upto)) + 1; // the run's start
			if (in_run)
				Cc |= (h == 32 ? 0xffffffffu : ((1u << h) - 1u)) << u;
		}
		on_row(token, u, starts, Tu, is_start, rem, h);
	}
}

// Quad record: plane, row, column, width-1, height-1, stream; then the quad's index among the
// plane's quads (all streams) and among the plane's quads of its stream.
__device__ __forceinline__ uint2 quad_record(int p, int u, int v, int w, int h, int st, uint32_t li, uint32_t lk) {
	return make_uint2((uint32_t)p | ((uint32_t)u << 8) | ((uint32_t)v << 13) | ((uint32_t)(w - 1) << 18) |
	                      ((uint32_t)(h - 1) << 23) | ((uint32_t)st << 28),
	                  li | (lk << 16));
}

// Record slot j: the first kQuadBuf in shared memory, then the CTA's global scratch; past both the
// records are dropped and misc[5] says so (the emission then merges again in windows).
__device__ __forceinline__ void put_record(Smem &S, uint32_t j, uint2 r) {
	if (j < (uint32_t)kQuadBuf)
		S.aux.quads[j] = r;
	else if (j - (uint32_t)kQuadBuf < S.spill_cap)
		S.spill[j - kQuadBuf] = r;
	else
		S.misc[5] = 1;
}
__device__ __forceinline__ uint2 get_record(const Smem &S, uint32_t j) {
	return j < (uint32_t)kQuadBuf ? S.aux.quads[j] : S.spill[j - kQuadBuf];
}

constexpr uint32_t kLonePlaneMin = 96; // faces of an all-lone plane emitted from its masks, at least

// Counts the quads of plane p (the calling warp) and keeps their records; misc[4] = records kept.
// A row none of whose cells equals the one below, below a row of which the same holds, is
// isolated: no quad of another row reaches it and its own quads do not grow down, so its quads are
// its horizontal runs (height 1) and its rows above and below scan as if it were not there. Lane u
// takes isolated row u, all at once; the exact row scan (warp_merge_plane) visits the other rows.
// A quad's index among the plane's quads (u-major, then v; all streams and per stream) counts the
// quads of the earlier rows of both kinds: isolated rows first give their per-row counts to the
// scan, whose per-row counts then place the isolated rows' quads.
__device__ void plane_count_one(Smem &S, int p) {
	const int lane = threadIdx.x & 31;
	const uint32_t lt = (1u << lane) - 1u;
	const uint32_t(*m)[4] = S.u.masks[p];
	const uint32_t rN = m[lane][0], rE = m[lane][1], rD = m[lane][2], rT = m[lane][3];
	{ // a plane of many faces that are all lone (a checkerboard's): its quads are its faces in
	  // u-major order, and the emission takes them straight from the visible and transparent-pass
	  // masks, a warp per plane, instead of from records (a few lone faces stay with the records,
	  // whose emission is spread over the whole CTA)
		const uint32_t rNu = __shfl_up_sync(0xffffffffu, rN, 1), rNd = __shfl_down_sync(0xffffffffu, rN, 1);
		const uint32_t lone = rN & ~(rN << 1) & ~(rN >> 1) & ~(lane == 0 ? 0u : rNu) & ~(lane == 31 ? 0u : rNd);
		const uint32_t all = __reduce_add_sync(0xffffffffu, __popc(rN));
		if (all >= kLonePlaneMin && __all_sync(0xffffffffu, lone == rN)) {
			const uint32_t tr = __reduce_add_sync(0xffffffffu, __popc(rN & rT));
			if (lane == 0) {
				S.seg_cnt[0][1 + p] = all - tr;
				S.seg_cnt[1][1 + p] = tr;
				atomicOr(&S.lone_planes[p >> 5], 1u << (p & 31));
			}
			return;
		}
	}
	const uint32_t rDup = __shfl_up_sync(0xffffffffu, rD, 1);
	const bool iso = rD == 0 && (lane == 0 || rDup == 0);
	const uint32_t icont = rN & (rN << 1) & (rE << 1); // bit v continues the run of v - 1
	const uint32_t istarts = iso ? (rN & ~icont) : 0u;
	// per row: quads (low half) and transparent-stream quads (high half), isolated rows only
	uint32_t itot;
	const uint32_t iexcl = warp_excl_scan((uint32_t)__popc(istarts) | ((uint32_t)__popc(istarts & rT) << 16), &itot);
	uint32_t ibase = 0;
	if (lane == 0 && (itot & 0xffffu))
		ibase = atomicAdd(&S.misc[4], itot & 0xffffu);
	ibase = __shfl_sync(0xffffffffu, ibase, 0);

	const uint32_t scanned = __ballot_sync(0xffffffffu, !iso && rN != 0); // rows for the row scan
	uint32_t b_all = 0, b_st[2] = {0, 0}; // quads of the scanned rows so far
	uint32_t mine = 0;                    // lane u: quads of scanned row u (packed like iexcl)
	const auto reserve = [&](uint32_t starts) {
		uint32_t b = 0;
		if (lane == 0)
			b = atomicAdd(&S.misc[4], (uint32_t)__popc(starts));
		return b;
	};
	warp_merge_plane(m, reserve, [&](uint32_t b, int u, uint32_t starts, uint32_t tmask, bool is_start, int w, int h) {
		const uint32_t cnt = __popc(starts), c1 = __popc(starts & tmask);
		const uint32_t base = __shfl_sync(0xffffffffu, b, 0);
		const uint32_t ex = __shfl_sync(0xffffffffu, iexcl, u); // isolated quads of the rows above u
		if (is_start) {
			const int st = (int)((tmask >> lane) & 1u);
			const uint32_t same = st ? (starts & tmask) : (starts & ~tmask);
			const uint32_t ex_all = ex & 0xffffu, ex_t = ex >> 16;
			const uint32_t li = ex_all + b_all + __popc(starts & lt);
			const uint32_t lk = (st ? ex_t + b_st[1] : ex_all - ex_t + b_st[0]) + __popc(same & lt);
			put_record(S, base + __popc(starts & lt), quad_record(p, u, lane, w, h, st, li, lk));
		}
		if (lane == u)
			mine = cnt | (c1 << 16);
		b_all += cnt;
		b_st[1] += c1;
		b_st[0] += cnt - c1;
	}, scanned);

	// the isolated rows' quads. Rows with many quads (a checkerboard's 16) are taken row by row,
	// lane = column, so that a row's records are written by one coalesced store; otherwise lane =
	// row, each lane walking its row's few quads.
	uint32_t btot;
	const uint32_t e = iexcl + (scanned ? warp_excl_scan(mine, &btot) : 0u);
	const uint32_t j = ibase + (iexcl & 0xffffu); // the row's first record slot
	const uint32_t irows = __ballot_sync(0xffffffffu, istarts != 0);
	if ((itot & 0xffffu) >= 12u * (uint32_t)__popc(irows)) {
		for (uint32_t rows_left = irows; rows_left; rows_left &= rows_left - 1u) {
			const int u = __ffs(rows_left) - 1;
			const uint32_t su = __shfl_sync(0xffffffffu, istarts, u), cu = __shfl_sync(0xffffffffu, icont, u);
			const uint32_t tu = __shfl_sync(0xffffffffu, rT, u), eu = __shfl_sync(0xffffffffu, e, u);
			const uint32_t ju = __shfl_sync(0xffffffffu, j, u);
			if ((su >> lane) & 1u) {
				const uint32_t e_all = eu & 0xffffu, e_t = eu >> 16;
				const uint32_t k_all = __popc(su & lt), k_t = __popc(su & tu & lt); // the row's quads before it
				const uint32_t after = lane == 31 ? 0u : (cu >> (lane + 1));
				const int w = __ffs(~after); // cells from this column to the end of its run
				const int st = (int)((tu >> lane) & 1u);
				const uint32_t lk = st ? e_t + k_t : e_all - e_t + (k_all - k_t);
				put_record(S, ju + k_all, quad_record(p, u, lane, w, 1, st, e_all + k_all, lk));
			}
		}
	} else {
		const uint32_t e_all = e & 0xffffu, e_t = e >> 16;
		uint32_t k_all = 0, k_t = 0;
		for (uint32_t rest = istarts; rest; rest &= rest - 1u) {
			const int v = __ffs(rest) - 1;
			const uint32_t after = v == 31 ? 0u : (icont >> (v + 1));
			const int w = __ffs(~after); // cells from v to the end of its run
			const int st = (int)((rT >> v) & 1u);
			const uint32_t lk = st ? e_t + k_t : e_all - e_t + (k_all - k_t);
			put_record(S, j + k_all, quad_record(p, lane, v, w, 1, st, e_all + k_all, lk));
			++k_all;
			k_t += (uint32_t)st;
		}
	}
	if (lane == 0) {
		const uint32_t t1 = (itot >> 16) + b_st[1];
		S.seg_cnt[0][1 + p] = (itot & 0xffffu) - (itot >> 16) + b_st[0];
		S.seg_cnt[1][1 + p] = t1;
	}
}

// Writes quad (u, v, w, h) of plane p: stream st, stream index k, all-stream index g. Called by all
// lanes of a warp; lanes without a quad (valid false) only take part in the box reduction.
__device__ void emit_plane_quad(Smem &S, const Emit &E, BoxAcc &box, bool valid, int p, int u, int v, int w, int h,
                                int st, uint32_t k, uint32_t g) {
	uint32_t mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
	if (valid) {
		const int a = p / 66, s = (p % 66) >> 1, inv = p & 1;
		const bool uv_cycle = a != 2; // (U + 1) % 3 == V for the YZX swizzle (BlockMeshAlgo.hpp:384)
		uint16_t t;
		Light4 l;
		face_key(S, a, s, inv, u, v, &t, &l);
		// vertex word 0 (x | y << 10 | z << 20 | axis << 30, positions in 1/16 voxel) of the first
		// corner, then the packed steps along the quad's two edges: the fields never carry into each
		// other (positions stay within 0..512)
		int ox, oy, oz;
		to_xyz(a, s, u, v, ox, oy, oz);
		const uint32_t w0 = ((uint32_t)ox << 4) | ((uint32_t)oy << 14) | ((uint32_t)oz << 24) | ((uint32_t)a << 30);
		const int shu = a == 1 ? 20 : 10, shv = a == 0 ? 20 : 0; // U and V fields: (y, z), (z, x), (y, x)
		const uint32_t hv = (uint32_t)h << (4 + shu), wv = (uint32_t)w << (4 + shv);
		const bool hfirst = (inv != 0) != uv_cycle;
		const uint32_t du = hfirst ? hv : wv, dv = hfirst ? wv : hv;
		const uint32_t face = (uint32_t)(2 * a + inv);
		const uint32_t w1 = ((uint32_t)(t & 0x1fffu) - 1u) | ((uint32_t)(t >> 13) << 10) | (face << 13);
		const uint32_t p0[4] = {w0, w0 + du, w0 + du + dv, w0 + dv};
		uint2 vt[4];
#pragma unroll
		for (int c = 0; c < 4; ++c)
			vt[c] = make_uint2(p0[c], w1 | (ao_get(l.ao, c) << 16) | (l4_get(l.sun, c) << 18) | (l4_get(l.torch, c) << 24));
		mn[0] = w0 & 1023u, mn[1] = (w0 >> 10) & 1023u, mn[2] = (w0 >> 20) & 1023u;
		mx[0] = p0[2] & 1023u, mx[1] = (p0[2] >> 10) & 1023u, mx[2] = (p0[2] >> 20) & 1023u;
		put_quad(S, E, st, k, g, vt, flip_of(l));
	}
	box_add_warp(S, box, valid, st, k / kQuadsPerMesh, mn, mx);
}

__device__ __forceinline__ void emit_record(Smem &S, const Emit &E, BoxAcc &box, bool valid, uint2 r) {
	const int p = (int)(r.x & 255u), st = (int)((r.x >> 28) & 1u);
	const uint32_t li = r.y & 0xffffu, lk = r.y >> 16;
	emit_plane_quad(S, E, box, valid, p, (int)((r.x >> 8) & 31u), (int)((r.x >> 13) & 31u), (int)((r.x >> 18) & 31u) + 1,
	                (int)((r.x >> 23) & 31u) + 1, st, valid ? S.seg_base[st][1 + p] + lk : 0u,
	                valid ? S.seg_base[2][1 + p] + li : 0u);
}

// Emits the quads of a plane all of whose faces are lone (the calling warp): each face is a quad of
// its own, its index among the plane's quads is its index among the plane's faces (u-major) and
// its stream the face's transparent-pass bit. Faces are taken in batches of whole rows, one per lane.
__device__ void emit_lone_plane(Smem &S, const Emit &E, BoxAcc &box, int p) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t(*m)[4] = S.u.masks[p];
	const uint32_t rN = m[lane][0], rT = m[lane][3] & m[lane][0];
	const uint32_t cnt = __popc(rN), incl = row_scan(cnt), start = incl - cnt;
	const uint32_t tcnt = __popc(rT), tstart = row_scan(tcnt) - tcnt;
	const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
	const uint32_t base_all = S.seg_base[2][1 + p], base_st[2] = {S.seg_base[0][1 + p], S.seg_base[1][1 + p]};
	const uint32_t upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
	uint32_t b = 0;
	int ub = 0;
	while (b < total) {
		// rows [ub, ue) whose faces fit in 32 lanes from index b (as in the key pass)
		const uint32_t over = __ballot_sync(0xffffffffu, lane >= ub && incl > b + 32);
		const int ue = over ? __ffs(over) - 1 : 32;
		const uint32_t be = __shfl_sync(0xffffffffu, start, ue & 31);
		const uint32_t bend = ue < 32 ? be : total;
		const uint32_t f = b + lane;
		const bool has = f < bend;
		const bool rin = lane >= ub && lane < ue && cnt > 0;
		const uint32_t M = __reduce_or_sync(0xffffffffu, rin ? 1u << (start - b) : 0u);
		if (rin)
			S.row_of[warp][start - b] = (uint8_t)lane;
		__syncwarp();
		const int u = has ? S.row_of[warp][31 - __clz(M & upto)] : 0;
		__syncwarp();
		const uint32_t su = __shfl_sync(0xffffffffu, start, u), Nu = __shfl_sync(0xffffffffu, rN, u);
		const uint32_t Tu = __shfl_sync(0xffffffffu, rT, u), tsu = __shfl_sync(0xffffffffu, tstart, u);
		const int v = has ? nth_set_bit(Nu, f - su) : 0;
		const int st = (int)((Tu >> v) & 1u);
		const uint32_t tb = tsu + __popc(Tu & ((1u << v) - 1u)); // transparent faces before this one
		const uint32_t lk = st ? tb : f - tb;
		emit_plane_quad(S, E, box, has, p, u, v, 1, 1, st, has ? base_st[st] + lk : 0u, has ? base_all + f : 0u);
		b = bend;
		ub = ue;
	}
}

// Emits the plane quads this CTA owns. Normally plane_count_one kept all their records; otherwise
// this CTA's quads are taken in windows of kQuadBuf (its planes in the order it took them, each
// plane's quads in order), the planes overlapping a window merge again to stage that window's
// records, and the whole CTA writes them. Emission of a window is spread over every thread: a
// heavy plane does not wait on the warp that merges it.
__device__ void planes_emit(Smem &S, const Emit &E, const Split &sp) {
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	BoxAcc box;
	if (!S.misc[5]) {
		const uint32_t n = S.misc[4];
		for (uint32_t j0 = (uint32_t)warp * 32; j0 < n; j0 += kThreads) {
			const uint32_t j = j0 + lane;
			emit_record(S, E, box, j < n, j < n ? get_record(S, j) : make_uint2(0, 0));
		}
		// then the planes whose faces are all lone, one warp per plane
		uint32_t any_lone = 0;
#pragma unroll
		for (int i = 0; i < (kPlanes + 31) / 32; ++i)
			any_lone |= S.lone_planes[i];
		const int n_mine = any_lone ? (int)S.misc[kMine] : 0;
		for (;;) {
			int j = 0;
			if (lane == 0)
				j = (int)atomicAdd(&S.misc[kClaimLone], 1u);
			j = __shfl_sync(0xffffffffu, j, 0);
			if (j >= n_mine)
				break;
			const int p = S.mine[j];
			if ((S.lone_planes[p >> 5] >> (p & 31)) & 1u)
				emit_lone_plane(S, E, box, p);
		}
		box_flush(S, box);
		return;
	}
	// own-quad offset of each taken plane (one warp; up to kPlanes entries)
	const int n_mine = (int)S.misc[kMine];
	__shared__ uint32_t s_obase[kPlanes + 1];
	if (warp == 0) {
		uint32_t run = 0;
		for (int j0 = 0; j0 < n_mine; j0 += 32) {
			const int j = j0 + lane;
			const int p = j < n_mine ? S.mine[j] : 0;
			const uint32_t c = j < n_mine ? S.seg_cnt[0][1 + p] + S.seg_cnt[1][1 + p] : 0u;
			uint32_t incl = c;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
				if (lane >= d)
					incl += o;
			}
			if (j < n_mine)
				s_obase[j] = run + incl - c;
			run += __shfl_sync(0xffffffffu, incl, 31);
		}
		if (lane == 0)
			s_obase[n_mine] = run;
	}
	__syncthreads();
	const uint32_t lt = (1u << lane) - 1u;
	const uint32_t own_quads = s_obase[n_mine];
	for (uint32_t w0 = 0; w0 < own_quads; w0 += kQuadBuf) {
		for (int jp = warp; jp < n_mine; jp += kWarps) {
			const int p = S.mine[jp];
			const uint32_t pb = s_obase[jp], pc = s_obase[jp + 1] - pb;
			if (!pc || pb >= w0 + kQuadBuf || pb + pc <= w0)
				continue;
			uint32_t n_all = 0, n_st[2] = {0, 0};
			warp_merge_plane(S.u.masks[p], [](uint32_t) { return 0u; },
			                 [&](uint32_t, int u, uint32_t starts, uint32_t tmask, bool is_start, int w, int h) {
				if (is_start) {
					const int st = (int)((tmask >> lane) & 1u);
					const uint32_t same = st ? (starts & tmask) : (starts & ~tmask);
					const uint32_t li = n_all + __popc(starts & lt), lk = n_st[st] + __popc(same & lt);
					const uint32_t i = pb + li;
					if (i >= w0 && i < w0 + kQuadBuf)
						S.aux.quads[i - w0] = quad_record(p, u, lane, w, h, st, li, lk);
				}
				n_all += __popc(starts);
				n_st[1] += __popc(starts & tmask);
				n_st[0] += __popc(starts & ~tmask);
			});
		}
		__syncthreads();
		const uint32_t n = min((uint32_t)kQuadBuf, own_quads - w0);
		for (uint32_t j0 = (uint32_t)warp * 32; j0 < n; j0 += kThreads) {
			const uint32_t j = j0 + lane;
			emit_record(S, E, box, j < n, j < n ? S.aux.quads[j] : make_uint2(0, 0));
		}
		__syncthreads();
	}
	box_flush(S, box);
}

// --------------------------------------------------------------------------------------- scans

// Exclusive scan of (a, b) over the CTA in thread order; totals returned to every thread.
__device__ void block_scan2(Smem &S, uint32_t a, uint32_t b, uint32_t &ea, uint32_t &eb, uint32_t &ta, uint32_t &tb) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t ia = a, ib = b;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const uint32_t xa = __shfl_up_sync(0xffffffffu, ia, d), xb = __shfl_up_sync(0xffffffffu, ib, d);
		if (lane >= d)
			ia += xa, ib += xb;
	}
	if (lane == 31)
		S.warp_sum[0][warp] = ia, S.warp_sum[1][warp] = ib;
	__syncthreads();
	if (warp == 0) {
		uint32_t wa = lane < kWarps ? S.warp_sum[0][lane] : 0, wb = lane < kWarps ? S.warp_sum[1][lane] : 0;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint32_t xa = __shfl_up_sync(0xffffffffu, wa, d), xb = __shfl_up_sync(0xffffffffu, wb, d);
			if (lane >= d)
				wa += xa, wb += xb;
		}
		if (lane < kWarps)
			S.warp_sum[0][lane] = wa, S.warp_sum[1][lane] = wb; // inclusive
	}
	__syncthreads();
	const uint32_t pa = warp ? S.warp_sum[0][warp - 1] : 0, pb = warp ? S.warp_sum[1][warp - 1] : 0;
	ea = pa + ia - a;
	eb = pb + ib - b;
	ta = S.warp_sum[0][kWarps - 1];
	tb = S.warp_sum[1][kWarps - 1];
	__syncthreads();
}

// Exclusive prefix of the per-segment counts in output order (custom, then planes 0..197): one
// thread per segment, a warp scan each, then the warp totals. Called by every thread; the caller
// syncs before reading the result.
__device__ void segment_scan(Smem &S) {
	constexpr int kScanWarps = (kSegments + 31) / 32;
	static_assert(kScanWarps <= kWarps, "one thread per segment");
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const bool in = tid < kSegments;
	const uint32_t so = in ? S.seg_cnt[0][tid] : 0u, stt = in ? S.seg_cnt[1][tid] : 0u;
	uint32_t io = so, it = stt;
	if (warp < kScanWarps) {
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint32_t xo = __shfl_up_sync(0xffffffffu, io, d), xt = __shfl_up_sync(0xffffffffu, it, d);
			if (lane >= d)
				io += xo, it += xt;
		}
		if (lane == 31)
			S.warp_sum[0][warp] = io, S.warp_sum[1][warp] = it;
	}
	__syncthreads();
	if (in) {
		uint32_t bo = io - so, bt = it - stt;
		for (int w = 0; w < warp; ++w)
			bo += S.warp_sum[0][w], bt += S.warp_sum[1][w];
		S.seg_base[0][tid] = bo;
		S.seg_base[1][tid] = bt;
		S.seg_base[2][tid] = bo + bt;
		if (tid == kSegments - 1) {
			S.misc[0] = bo + so; // opaque quads
			S.misc[1] = bt + stt; // transparent quads
		}
	}
}

// ------------------------------------------------------------------------------- whole chunk

// Where a chunk's meshes go: an arena shared by a batch (cursors advanced atomically), or the
// single-chunk buffers (cursors reset to zero before the launch).
struct Arena {
	uint2 *verts;
	uint16_t *idx;
	hc_mesh_desc *meshes;
	unsigned long long *quad_cursor;
	unsigned int *mesh_cursor;
	unsigned long long quad_cap;
	unsigned int mesh_cap;
	uint32_t *results;     // per batch position: opaque quads, transparent quads, first mesh, mesh count, status
	uint2 *spill = nullptr; // kSpillRecs quad records per CTA of the grid (blockIdx.x), or null
};

enum : uint32_t { kChunkOk = 0, kChunkCapacity = 1 };

// Relights and meshes one chunk whose 27 neighbour pointers are already in S.blk / S.hgt / S.pln
// (and S.lvl / S.edg). With sp.c > 1 the c CTAs of a cluster mesh it together: each stages it, owns a
// share of the face planes, and they exchange per-plane counts, the arena reservation and the
// meshes' bounding boxes through distributed shared memory; CTA 0 writes the results and the
// mesh descriptors. Every CTA of the cluster must call this with the same chunk.
__device__ void mesh_chunk_cta(Smem &S, const DevTables &T, const Arena &A, uint32_t pos, Split sp = Split{1, 0}) {
	namespace cg = cooperative_groups;
	const int tid = threadIdx.x;
	const bool lead = sp.rank == 0;
	for (int i = tid; i < 2 * kMaxMeshesPerStream; i += kThreads) {
		uint32_t *bb = S.aabb[i / kMaxMeshesPerStream][i % kMaxMeshesPerStream];
		bb[0] = bb[1] = bb[2] = 0xffffffffu;
		bb[3] = bb[4] = bb[5] = 0u;
		S.trig[i / kMaxMeshesPerStream][i % kMaxMeshesPerStream] = 0xffffffffu;
	}
	for (int i = tid; i < 2 * (kSegments + 1); i += kThreads)
		S.seg_cnt[i / (kSegments + 1)][i % (kSegments + 1)] = 0;
	if (tid < 5) // the claim counters, records kept, records overflow; the stage's barriers (and,
	             // in a cluster, the relight's) order this before any CTA's plane phases
		S.misc[tid < 3 ? kClaimKeys + tid : tid + 1] = 0; // misc[13..15], misc[4..5]
	if (tid < (kPlanes + 31) / 32)
		S.lone_planes[tid] = 0;
	if (tid == 0) {
		S.spill = A.spill ? A.spill + (size_t)blockIdx.x * kSpillRecs : nullptr;
		S.spill_cap = A.spill ? kSpillRecs : 0u;
	}
	bool has_custom;
	const bool blank = stage_classes(S, T, has_custom);

	uint32_t qo = 0, qt = 0;
	uint32_t eo = 0, et = 0;
	if (!blank) {
		uint32_t co = 0, ct = 0, to, tt;
		if (lead && has_custom) // no inner block with a custom mesh: nothing to count
			custom_count(S, tid * kBlocksPerThread, co, ct);
		block_scan2(S, co, ct, eo, et, to, tt);
		if (!S.lvl[26])
			relight_window(S, T, sp); // the relight scratch shares memory with the plane masks
		else if (!S.pln[26])
			light_from_levels(S); // with chunk planes the staging decoded the light
		__syncthreads();
		plane_visibility(S);
		__syncthreads();
		const int live = order_planes(S);
		const int nsplit = sp.c > 1 ? 0 : split_heavy_planes(S, live);
		if (sp.c > 1) // CTA 0's plane counter was reset for this chunk before any CTA takes from it
			cooperative_groups::this_cluster().sync();
		plane_keys(S, sp, live, nsplit); // with each plane's quad count and records
		if (tid == 0) {
			S.seg_cnt[0][0] = to;
			S.seg_cnt[1][0] = tt;
		}
		__syncthreads();
		if (sp.c > 1) { // every CTA takes the counts of the segments the others own
			cg::cluster_group cl = cg::this_cluster();
			cl.sync();
			for (int i = tid; i < kSegments; i += kThreads) {
				const int owner = i == 0 ? 0 : cl.map_shared_rank(&S.plane_owner[0], 0)[i - 1];
				if (owner != sp.rank) {
					const uint32_t *src = cl.map_shared_rank(&S.seg_cnt[0][0], owner);
					S.seg_cnt[0][i] = src[i];
					S.seg_cnt[1][i] = src[(kSegments + 1) + i];
				}
			}
			__syncthreads();
		}
		segment_scan(S);
		__syncthreads();
		qo = S.misc[0];
		qt = S.misc[1];
	}

	const uint32_t q = qo + qt;
	const uint32_t mo = (qo + kQuadsPerMesh - 1) / kQuadsPerMesh, mt = (qt + kQuadsPerMesh - 1) / kQuadsPerMesh;
	if (lead && tid == 0) {
		const unsigned long long q0 = q ? atomicAdd(A.quad_cursor, (unsigned long long)q) : 0ull;
		const unsigned int m0 = (mo + mt) ? atomicAdd(A.mesh_cursor, mo + mt) : 0u;
		const uint32_t status = (q0 + q > A.quad_cap || m0 + mo + mt > A.mesh_cap) ? kChunkCapacity : kChunkOk;
		S.misc[8] = (uint32_t)q0, S.misc[9] = (uint32_t)(q0 >> 32), S.misc[10] = m0, S.misc[11] = status;
		uint32_t *r = A.results + 5 * pos;
		r[0] = qo, r[1] = qt, r[2] = m0, r[3] = mo + mt, r[4] = status;
	}
	if (sp.c > 1 && !blank) { // the reservation of CTA 0
		cg::cluster_group cl = cg::this_cluster();
		cl.sync();
		if (!lead && tid < 4)
			S.misc[8 + tid] = cl.map_shared_rank(&S.misc[0], 0)[8 + tid];
	}
	__syncthreads();
	const unsigned long long q0 = (unsigned long long)S.misc[8] | ((unsigned long long)S.misc[9] << 32);
	const unsigned int m0 = S.misc[10];
	if (blank || q == 0 || S.misc[11] != kChunkOk)
		return;

	const Emit E{A.verts, A.idx, q0, qo};
	if (lead && has_custom)
		custom_emit(S, E, tid * kBlocksPerThread, eo, et, eo + et);
	planes_emit(S, E, sp);
	__syncthreads(); // every quad's box and closing position is in before the descriptors are written

	if (sp.c > 1) { // CTA 0 merges the boxes and closing positions of every CTA's quads
		cg::cluster_group cl = cg::this_cluster();
		cl.sync();
		if (lead)
			for (int i = tid; i < 2 * kMaxMeshesPerStream; i += kThreads) {
				const int st = i / kMaxMeshesPerStream, m = i % kMaxMeshesPerStream;
				uint32_t *bb = S.aabb[st][m];
				for (int r = 1; r < sp.c; ++r) {
					const uint32_t *o = cl.map_shared_rank(&S.aabb[st][m][0], r);
					bb[0] = min(bb[0], o[0]), bb[1] = min(bb[1], o[1]), bb[2] = min(bb[2], o[2]);
					bb[3] = max(bb[3], o[3]), bb[4] = max(bb[4], o[4]), bb[5] = max(bb[5], o[5]);
					S.trig[st][m] = min(S.trig[st][m], cl.map_shared_rank(&S.trig[st][m], r)[0]);
				}
			}
		__syncthreads();
	}

	// Mesh descriptors: closed meshes in closing order, then the open opaque and transparent ones.
	if (lead && tid == 0) {
		uint32_t io = 0, it = 0, out = m0;
		const auto put = [&](int st, uint32_t j, uint32_t nst) {
			const uint32_t first = j * kQuadsPerMesh, n = min((uint32_t)kQuadsPerMesh, nst - first);
			const unsigned long long fq = q0 + (st ? qo : 0u) + first;
			hc_mesh_desc d;
			d.vertex_offset = (uint32_t)(4 * fq);
			d.vertex_count = 4 * n;
			d.index_offset = (uint32_t)(6 * fq);
			d.index_count = 6 * n;
			for (int c = 0; c < 3; ++c) {
				d.aabb_min[c] = S.aabb[st][j][c];
				d.aabb_max[c] = S.aabb[st][j][3 + c];
			}
			d.transparent = (uint32_t)st;
			d.chunk = pos;
			A.meshes[out++] = d;
		};
		while (io + 1 < mo || it + 1 < mt) {
			const bool take_o = it + 1 >= mt || (io + 1 < mo && S.trig[0][io] < S.trig[1][it]);
			if (take_o)
				put(0, io, qo), ++io;
			else
				put(1, it, qt), ++it;
		}
		if (mo)
			put(0, mo - 1, qo);
		if (mt)
			put(1, mt - 1, qt);
	}
}

} // namespace hc
