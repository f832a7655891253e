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
// A warp builds them row by row with ballots; one thread then runs the exact sequential greedy
// scan on the masks with word operations. Counts per (stream, segment) are prefix-summed in
// output order, which gives every quad its final stream index k before anything is written, so
// all quads are written in parallel straight to their reference positions.
#pragma once
#include "hc_relight.cuh"

namespace hc {

struct Emit {
	uint2 *verts;
	uint16_t *idx;
	unsigned long long q0; // first quad of this chunk in the arena
	uint32_t qo;           // opaque quads (the transparent stream starts after them)
};

__device__ __forceinline__ void put_quad(Smem &S, const Emit &E, int st, uint32_t k, uint32_t g, const uint2 v[4], bool flip,
                                         const uint32_t mn[3], const uint32_t mx[3]) {
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
	uint32_t *bb = S.aabb[st][m];
	atomicMin(bb + 0, mn[0]), atomicMin(bb + 1, mn[1]), atomicMin(bb + 2, mn[2]);
	atomicMax(bb + 3, mx[0]), atomicMax(bb + 4, mx[1]), atomicMax(bb + 5, mx[2]);
	if (k > 0 && r == 0)
		S.trig[st][m - 1] = g;
}

// ------------------------------------------------------------------------------------- staging

__device__ void stage_classes(Smem &S, const DevTables &T) {
	for (int i = threadIdx.x; i < 256; i += kThreads)
		S.classes[i] = T.classes[i];
	for (int i = threadIdx.x; i < kClsCells; i += kThreads) {
		const int x = i % kClsX - 2, z = (i / kClsX) % kClsZ - 2, y = i / (kClsX * kClsZ) - 1;
		S.cls[i] = __ldg(T.class_of + raw_at(S, x, y, z));
	}
}

// True when the chunk can produce no quad: every inner block has no texture and no custom mesh,
// or every inner block and every block of the six adjacent layers is an opaque full cube.
__device__ bool chunk_is_blank(Smem &S) {
	bool content = false, open = false;
	for (int i = threadIdx.x; i < kClsCells; i += kThreads) {
		const int x = i % kClsX - 2, z = (i / kClsX) % kClsZ - 2, y = i / (kClsX * kClsZ) - 1;
		const int out = (x < 0 || x >= kChunk) + (y < 0 || y >= kChunk) + (z < 0 || z >= kChunk);
		const uint8_t f = S.classes[S.cls[i]].flags;
		if (out == 0) {
			content |= !(f & kFEmpty);
			open |= !(f & kFOpaqueCube);
		} else if (out == 1 && x >= -1 && x <= kChunk && z >= -1 && z <= kChunk) {
			open |= !(f & kFOpaqueCube);
		}
	}
	content = __syncthreads_or(content);
	open = __syncthreads_or(open);
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

// Stream counts of the custom faces of inner blocks [first, first + 64).
__device__ void custom_count(const Smem &S, int first, uint32_t &co, uint32_t &ct) {
	co = ct = 0;
	for (int i = first; i < first + 64; ++i) {
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
	for (int i = first; i < first + 64; ++i) {
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
				if (S.classes[class_at(S, ne[0], ne[1], ne[2])].flags & kFIndirect)
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
			put_quad(S, E, st, st ? kt : ko, g, v, true, mn, mx);
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

// Pass 1: visible and transparent-pass masks of both planes of every slice (no light needed).
// Returns true if any face of the chunk is visible.
__device__ bool plane_visibility(Smem &S) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	bool any = false;
	for (int sl = warp; sl < kSlices; sl += kWarps) {
		const int a = sl / 33, s = sl - a * 33;
		uint32_t(*mA)[4] = S.u.masks[plane_id(a, s, 0)];
		uint32_t(*mB)[4] = S.u.masks[plane_id(a, s, 1)];
		for (int u = 0; u < 32; ++u) {
			int x, y, z;
			to_xyz(a, s, u, lane, x, y, z);
			int nx = x, ny = y, nz = z;
			(a == 0 ? nx : (a == 1 ? ny : nz)) -= 1;
			const uint16_t ta = get_tex(S, nx, ny, nz, 2 * a), tb = get_tex(S, x, y, z, 2 * a + 1);
			const bool va = s != 0 && show(ta, tb), vb = s != 32 && show(tb, ta);
			const uint32_t NA = __ballot_sync(0xffffffffu, va), NB = __ballot_sync(0xffffffffu, vb);
			const uint32_t TA = __ballot_sync(0xffffffffu, va && tex_transpass(ta));
			const uint32_t TB = __ballot_sync(0xffffffffu, vb && tex_transpass(tb));
			if (lane == 0) {
				mA[u][0] = NA, mA[u][1] = 0, mA[u][2] = 0, mA[u][3] = TA;
				mB[u][0] = NB, mB[u][1] = 0, mB[u][2] = 0, mB[u][3] = TB;
			}
			any |= (NA | NB) != 0;
		}
	}
	return __syncthreads_or(any);
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

// Pass 2 (after relight): equal-to-right and equal-to-below masks of both planes of every slice.
__device__ void plane_keys(Smem &S) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int sl = warp; sl < kSlices; sl += kWarps) {
		const int a = sl / 33, s = sl - a * 33;
#pragma unroll
		for (int inv = 0; inv < 2; ++inv) {
			uint32_t(*m)[4] = S.u.masks[plane_id(a, s, inv)];
			Key prev{0, 0, 0};
			bool prev_vis = false;
			for (int u = 0; u < 32; ++u) {
				const uint32_t N = m[u][0];
				if (!N) { // nothing visible: no run continues here and nothing matches the row above
					if (lane == 0) {
						m[u][1] = 0;
						if (u > 0)
							m[u - 1][2] = 0;
					}
					prev_vis = false;
					continue;
				}
				const bool vis = (N >> lane) & 1u;
				Key k{0, 0, 0};
				if (vis)
					k = face_key(S, a, s, inv, u, lane, nullptr, nullptr);
				const Key right = shfl_down_key(k);
				const bool rv = lane < 31 && ((N >> (lane + 1)) & 1u);
				const uint32_t E = __ballot_sync(0xffffffffu, vis && rv && key_eq(k, right));
				const uint32_t D = __ballot_sync(0xffffffffu, vis && prev_vis && key_eq(k, prev));
				if (lane == 0) {
					m[u][1] = E;
					if (u > 0)
						m[u - 1][2] = D; // bit v: rows u-1 and u hold the same face key at column v
				}
				prev = k;
				prev_vis = vis;
			}
			if (lane == 0)
				m[31][2] = 0;
		}
	}
}

// Exact greedy scan of one plane from its masks (BlockMeshAlgo.hpp:345-477). on_quad(u, v, w, h, st)
// is called in the reference's order: row-major by the quad's first cell.
template <typename F> __device__ __forceinline__ void merge_plane(const uint32_t (*m)[4], F &&on_quad) {
	uint32_t consumed[32];
#pragma unroll
	for (int i = 0; i < 32; ++i)
		consumed[i] = 0;
	for (int u = 0; u < 32; ++u) {
		const uint32_t live = m[u][0] & ~consumed[u];
		if (!live)
			continue;
		const uint32_t cont = live & (live << 1) & (m[u][1] << 1); // bit v continues the run of v-1
		uint32_t starts = live & ~cont;
		const uint32_t tp = m[u][3];
		while (starts) {
			const int v = __ffs(starts) - 1;
			starts &= starts - 1;
			const uint32_t after = v == 31 ? 0u : (cont >> (v + 1));
			const int w = __ffs(~after);
			const uint32_t run = w == 32 ? 0xffffffffu : (((1u << w) - 1u) << v);
			int h = 1;
			while (u + h < 32 && (m[u + h - 1][2] & run) == run) {
				consumed[u + h] |= run;
				++h;
			}
			on_quad(u, v, w, h, (int)((tp >> v) & 1u));
		}
	}
}

__device__ void plane_count(Smem &S, int p) {
	uint32_t c[2] = {0, 0};
	merge_plane(S.u.masks[p], [&](int, int, int, int, int st) { ++c[st]; });
	S.seg_cnt[0][1 + p] = c[0];
	S.seg_cnt[1][1 + p] = c[1];
}

__device__ void plane_emit(Smem &S, const Emit &E, int p) {
	const int a = p / 66, s = (p % 66) >> 1, inv = p & 1;
	const bool uv_cycle = a != 2; // (U + 1) % 3 == V for the YZX swizzle (BlockMeshAlgo.hpp:384)
	uint32_t k[2] = {S.seg_base[0][1 + p], S.seg_base[1][1 + p]};
	uint32_t g = S.seg_base[2][1 + p];
	merge_plane(S.u.masks[p], [&](int u, int v, int w, int h, int st) {
		uint16_t t;
		Light4 l;
		face_key(S, a, s, inv, u, v, &t, &l);
		int o[3], hv[3], wv[3];
		to_xyz(a, s, u, v, o[0], o[1], o[2]);
		to_xyz(a, 0, h, 0, hv[0], hv[1], hv[2]);
		to_xyz(a, 0, 0, w, wv[0], wv[1], wv[2]);
		const bool hfirst = (inv != 0) != uv_cycle;
		const int *du = hfirst ? hv : wv, *dv = hfirst ? wv : hv;
		const uint32_t face = (uint32_t)(2 * a + inv);
		uint2 vt[4];
		const int cx[4] = {o[0], o[0] + du[0], o[0] + du[0] + dv[0], o[0] + dv[0]};
		const int cy[4] = {o[1], o[1] + du[1], o[1] + du[1] + dv[1], o[1] + dv[1]};
		const int cz[4] = {o[2], o[2] + du[2], o[2] + du[2] + dv[2], o[2] + dv[2]};
#pragma unroll
		for (int c = 0; c < 4; ++c)
			vt[c] = pack_vertex((uint32_t)cx[c] << 4, (uint32_t)cy[c] << 4, (uint32_t)cz[c] << 4, (uint32_t)a, face,
			                    ao_get(l.ao, c), l4_get(l.sun, c), l4_get(l.torch, c), t);
		const uint32_t mn[3] = {(uint32_t)cx[0] << 4, (uint32_t)cy[0] << 4, (uint32_t)cz[0] << 4};
		const uint32_t mx[3] = {(uint32_t)cx[2] << 4, (uint32_t)cy[2] << 4, (uint32_t)cz[2] << 4};
		put_quad(S, E, st, k[st], g, vt, flip_of(l), mn, mx);
		++k[st];
		++g;
	});
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

// Exclusive prefix of the per-segment counts in output order (custom, then planes 0..197).
__device__ void segment_scan(Smem &S) {
	if (threadIdx.x >= 32)
		return;
	const int lane = threadIdx.x;
	constexpr int kPer = (kSegments + 31) / 32;
	uint32_t so = 0, stt = 0;
	for (int i = 0; i < kPer; ++i) {
		const int sidx = lane * kPer + i;
		if (sidx < kSegments)
			so += S.seg_cnt[0][sidx], stt += S.seg_cnt[1][sidx];
	}
	uint32_t io = so, it = stt;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const uint32_t xo = __shfl_up_sync(0xffffffffu, io, d), xt = __shfl_up_sync(0xffffffffu, it, d);
		if (lane >= d)
			io += xo, it += xt;
	}
	uint32_t bo = io - so, bt = it - stt;
	for (int i = 0; i < kPer; ++i) {
		const int sidx = lane * kPer + i;
		if (sidx < kSegments) {
			S.seg_base[0][sidx] = bo;
			S.seg_base[1][sidx] = bt;
			S.seg_base[2][sidx] = bo + bt;
			bo += S.seg_cnt[0][sidx];
			bt += S.seg_cnt[1][sidx];
		}
	}
	if (lane == 31) {
		S.misc[0] = io; // opaque quads
		S.misc[1] = it; // transparent quads
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
	uint32_t *results; // per batch position: opaque quads, transparent quads, first mesh, mesh count, status
};

enum : uint32_t { kChunkOk = 0, kChunkCapacity = 1 };

// Relights and meshes one chunk whose 27 neighbour pointers are already in S.blk / S.hgt.
__device__ void mesh_chunk_cta(Smem &S, const DevTables &T, const Arena &A, uint32_t pos) {
	const int tid = threadIdx.x;
	stage_classes(S, T);
	for (int i = tid; i < 2 * kMaxMeshesPerStream; i += kThreads) {
		uint32_t *bb = S.aabb[i / kMaxMeshesPerStream][i % kMaxMeshesPerStream];
		bb[0] = bb[1] = bb[2] = 0xffffffffu;
		bb[3] = bb[4] = bb[5] = 0u;
	}
	__syncthreads();

	uint32_t qo = 0, qt = 0;
	uint32_t eo = 0, et = 0;
	if (!chunk_is_blank(S)) {
		uint32_t co, ct, to, tt;
		custom_count(S, tid * 64, co, ct);
		block_scan2(S, co, ct, eo, et, to, tt);
		relight_window(S, T); // the relight scratch shares memory with the plane masks
		__syncthreads();
		plane_visibility(S);
		__syncthreads();
		plane_keys(S);
		if (tid == 0) {
			S.seg_cnt[0][0] = to;
			S.seg_cnt[1][0] = tt;
		}
		__syncthreads();
		if (tid < kPlanes)
			plane_count(S, tid);
		__syncthreads();
		segment_scan(S);
		__syncthreads();
		qo = S.misc[0];
		qt = S.misc[1];
	}

	const uint32_t q = qo + qt;
	const uint32_t mo = (qo + kQuadsPerMesh - 1) / kQuadsPerMesh, mt = (qt + kQuadsPerMesh - 1) / kQuadsPerMesh;
	__shared__ unsigned long long s_q0;
	__shared__ unsigned int s_m0;
	__shared__ uint32_t s_status;
	if (tid == 0) {
		s_q0 = q ? atomicAdd(A.quad_cursor, (unsigned long long)q) : 0ull;
		s_m0 = (mo + mt) ? atomicAdd(A.mesh_cursor, mo + mt) : 0u;
		s_status = (s_q0 + q > A.quad_cap || s_m0 + mo + mt > A.mesh_cap) ? kChunkCapacity : kChunkOk;
	}
	__syncthreads();
	const unsigned long long q0 = s_q0;
	const unsigned int m0 = s_m0;
	if (tid == 0) {
		uint32_t *r = A.results + 5 * pos;
		r[0] = qo, r[1] = qt, r[2] = m0, r[3] = mo + mt, r[4] = s_status;
	}
	if (q == 0 || s_status != kChunkOk)
		return;

	const Emit E{A.verts, A.idx, q0, qo};
	custom_emit(S, E, tid * 64, eo, et, eo + et);
	if (tid < kPlanes)
		plane_emit(S, E, tid);
	__syncthreads();

	// Mesh descriptors: closed meshes in closing order, then the open opaque and transparent ones.
	if (tid == 0) {
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
