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

constexpr uint64_t kWinMask = (1ull << kWin) - 1ull;

// Distance of one coordinate to [-1, 33) as IsBorderLightInterfere computes it.
__device__ __forceinline__ int axis_dist(int v) { return v < -1 ? -1 - v : (v >= 33 ? v - 33 : 0); }

// Cells of window row (wy, wz) whose distance to the box is below t.
__device__ __forceinline__ uint64_t dist_mask(int t, int wy, int wz) {
	int rem = t - 1 - axis_dist(wy - 15) - axis_dist(wz - 15);
	if (rem < 0)
		return 0;
	int lo = 14 - rem, hi = 48 + rem;
	lo = lo < 0 ? 0 : lo;
	hi = hi > kWin - 1 ? kWin - 1 : hi;
	return ((~0ull) >> (63 - hi)) & ~((1ull << lo) - 1ull);
}

// Writes level `t` into the light nibble of newly lit cells of row (wy, wz) inside [-1, 32]^3.
__device__ __forceinline__ void write_new(uint8_t *light, int wy, int wz, uint64_t bits, uint32_t t, int shift) {
	if (wy < 14 || wy > 47 || wz < 14 || wz > 47)
		return;
	bits &= 0x0000ffffffffc000ull; // window x in [14, 47]  <=>  x in [-1, 32]
	const int row = ((wy - 14) * kLt + (wz - 14)) * kLt;
	while (bits) {
		int b = __ffsll((long long)bits) - 1;
		bits &= bits - 1;
		light[row + b - 14] |= (uint8_t)(t << shift);
	}
}

__device__ void relight_window(Smem &S, const DevTables &T) {
	Relight &R = S.u.rl;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	for (int i = tid; i < (kWinRows + 31) / 32; i += kThreads)
		R.low_rows[i] = 0;
	for (int i = tid; i < kLtCells; i += kThreads)
		S.light[i] = 0;
	__syncthreads();

	// Seeds and the pass mask, one warp per row, two 32-cell halves.
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
			R.sun[r] = sun;
			R.torch[r] = torch;
			if (low)
				atomicOr(&R.low_rows[r >> 5], 1u << (r & 31));
		}
	}
	__syncthreads();
	for (int r = tid; r < kWinRows; r += kThreads) {
		const int wy = r / kWin, wz = r - wy * kWin;
		write_new(S.light, wy, wz, R.sun[r], 15, 0);
		write_new(S.light, wy, wz, R.torch[r], 15, 4);
	}

	constexpr int kRowsPerThread = (kWinRows + kThreads - 1) / kThreads;
	for (int t = 14; t >= 1; --t) {
		uint64_t ns[kRowsPerThread], nt[kRowsPerThread];
#pragma unroll
		for (int k = 0; k < kRowsPerThread; ++k) {
			const int r = tid + k * kThreads;
			if (r >= kWinRows)
				continue;
			const int wy = r / kWin, wz = r - wy * kWin;
			const uint64_t cs = R.sun[r], ct = R.torch[r];
			ns[k] = cs, nt[k] = ct;
			const uint64_t m = R.pass[r] & dist_mask(t, wy, wz);
			if (m) {
				uint64_t ds = (cs << 1) | (cs >> 1), dt = (ct << 1) | (ct >> 1);
				if (wz > 0)
					ds |= R.sun[r - 1], dt |= R.torch[r - 1];
				if (wz < kWin - 1)
					ds |= R.sun[r + 1], dt |= R.torch[r + 1];
				if (wy > 0)
					ds |= R.sun[r - kWin], dt |= R.torch[r - kWin];
				if (wy < kWin - 1)
					ds |= R.sun[r + kWin], dt |= R.torch[r + kWin];
				ns[k] |= m & ds;
				nt[k] |= m & dt;
			}
			if ((R.low_rows[r >> 5] >> (r & 31)) & 1u) { // emitters of level t enter now
				const int y = wy - 15, z = wz - 15;
				for (int wx = 0; wx < kWin; ++wx)
					if (S.classes[__ldg(T.class_of + raw_at(S, wx - 15, y, z))].light == t)
						nt[k] |= 1ull << wx;
			}
		}
		__syncthreads();
#pragma unroll
		for (int k = 0; k < kRowsPerThread; ++k) {
			const int r = tid + k * kThreads;
			if (r >= kWinRows)
				continue;
			const int wy = r / kWin, wz = r - wy * kWin;
			const uint64_t gs = ns[k] & ~R.sun[r], gt = nt[k] & ~R.torch[r];
			if (gs) {
				R.sun[r] = ns[k];
				write_new(S.light, wy, wz, gs, (uint32_t)t, 0);
			}
			if (gt) {
				R.torch[r] = nt[k];
				write_new(S.light, wy, wz, gt, (uint32_t)t, 4);
			}
		}
		__syncthreads();
	}
}

} // namespace hc
