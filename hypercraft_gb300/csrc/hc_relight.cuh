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
#include "hc_device.cuh"

namespace hc {

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
__device__ void seed_from_planes(Smem &S) {
	Relight &R = S.u.rl;
	for (int r = threadIdx.x; r < kWinRows; r += kThreads) {
		const int wy = r / kWin, wz = r - wy * kWin, y = wy - 15, z = wz - 15;
		const int prow = (z & 31) + 32 * (y & 31);
		uint32_t w[3][3], low = 0;
#pragma unroll
		for (int c = 0; c < 3; ++c) {
			const uint32_t *P = S.pln[nb_index(c * 32 - 1, y, z)];
#pragma unroll
			for (int pl = 0; pl < 3; ++pl)
				w[c][pl] = __ldg(P + pl * kPlaneWords + prow);
			low |= __ldg(P + 3 * kPlaneWords + (prow >> 5)) >> (prow & 31);
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
__device__ void seed_from_blocks(Smem &S, const DevTables &T) {
	Relight &R = S.u.rl;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int r = warp; r < kWinRows; r += kWarps) {
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
	for (int r = threadIdx.x; r < kWinRows; r += kThreads) {
		const int wy = r / kWin, wz = r - wy * kWin;
		const ulonglong2 l = R.lit[r];
		write_row15(light_bytes(S), wy, wz, l.x, l.y);
	}
}

// Bit of row r in a row bitmap.
__device__ __forceinline__ bool row_bit(const uint32_t *m, int r) { return (m[r >> 5] >> (r & 31)) & 1u; }

__device__ void relight_window(Smem &S, const DevTables &T) {
	Relight &R = S.u.rl;
	const int tid = threadIdx.x;
	for (int i = tid; i < kRowWords; i += kThreads)
		R.low_rows[i] = 0, R.changed[0][i] = 0, R.changed[1][i] = 0;
	__syncthreads();
	if (S.pln[26])
		seed_from_planes(S);
	else
		seed_from_blocks(S, T);
	__syncthreads();

	// A row can gain cells at level t only when it or one of its four neighbour rows changed at
	// level t + 1: otherwise its dilation is the one it already saw, while the distance mask only
	// shrinks. So after the first level only rows next to the last changes (the light front) and
	// rows holding emitters of the level are visited.
	constexpr int kRowsPerThread = (kWinRows + kThreads - 1) / kThreads;
	int rem0[kRowsPerThread]; // t - 1 - dist(y, z) = t + rem0
#pragma unroll
	for (int k = 0; k < kRowsPerThread; ++k) {
		const int r = tid + k * kThreads;
		const int wy = r / kWin, wz = r - wy * kWin;
		rem0[k] = r < kWinRows ? -1 - axis_dist(wy - 15) - axis_dist(wz - 15) : -1000;
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
			const int r = tid + k * kThreads;
			const int rem = t + rem0[k];
			if (r >= kWinRows)
				continue;
			const bool low = row_bit(R.low_rows, r);
			if (rem < 0 && !low)
				continue;
			const int wy = r / kWin, wz = r - wy * kWin;
			if (t < 14 && !low) {
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
			const int r = tid + k * kThreads;
			const int wy = r / kWin, wz = r - wy * kWin;
			const ulonglong2 cur = R.lit[r];
			R.lit[r] = make_ulonglong2(ns[k], nt[k]);
			atomicOr(&cur_chg[r >> 5], 1u << (r & 31));
			write_new(light, wy, wz, ns[k] & ~cur.x, (uint32_t)t, 0);
			write_new(light, wy, wz, nt[k] & ~cur.y, (uint32_t)t, 4);
		}
		__syncthreads();
	}
}

// ------------------------------------------------------------------------------------ planes

// Bit planes of one 32-cell row (y, z) of a chunk: pass (transparency != opaque), sunlit
// (Chunk::GetSunlight) and emitters of level 15; returns whether the row holds an emitter of
// level 1..14. Uniform rows (one raw value) take one lookup.
__device__ __forceinline__ bool chunk_plane_row(const uint16_t *blk, const int8_t *hgt, const DevClass *classes,
                                                const uint8_t *class_of, int y, int z, uint32_t &pass, uint32_t &sun,
                                                uint32_t &t15) {
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
		const DevClass &k = classes[__ldg(class_of + (w0 & 0xffffu))];
		pass = (k.flags & kFIndirect) ? 0xffffffffu : 0u;
		t15 = k.light >= 15 ? 0xffffffffu : 0u;
		low = k.light > 0 && k.light < 15;
	} else {
#pragma unroll
		for (int i = 0; i < 4; ++i) {
			const uint32_t ws[4] = {q[i].x, q[i].y, q[i].z, q[i].w};
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const uint32_t raw = (ws[j >> 1] >> (16 * (j & 1))) & 0xffffu;
				const DevClass &k = classes[__ldg(class_of + raw)];
				const int x = 8 * i + j;
				pass |= (uint32_t)((k.flags & kFIndirect) != 0) << x;
				t15 |= (uint32_t)(k.light >= 15) << x;
				low |= k.light > 0 && k.light < 15;
			}
		}
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

} // namespace hc
