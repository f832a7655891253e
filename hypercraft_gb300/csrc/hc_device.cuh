// Device-side tables, shared-memory layout and small helpers of the GB300 chunk mesher.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>
#include <stdint.h>

#include "hc_flow.h"
#include "hc_registry.h"

namespace hc {

constexpr int kThreads = 1024;
constexpr int kBlocksPerThread = 32768 / kThreads; // inner blocks per thread in the custom-mesh passes
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 32;
constexpr int kQuadsPerMesh = 16383;       // 65,532 vertices: the uint16 split point (BlockMeshAlgo.hpp:274)
constexpr int kMaxMeshesPerStream = 48;    // > 720,896 / 16,383
constexpr int kMaxSplit = 16;              // face planes keyed in row parts per chunk, at most
constexpr int kMaxParts = 8;               // row parts of a split face plane, at most
constexpr int kPlanes = 198;               // 3 axes x 33 slices x 2 face directions
constexpr int kSlices = 99;
constexpr int kSegments = kPlanes + 1;     // segment 0 = custom meshes, then the planes in output order

// Staged block classes cover [-1, 32]^3, the cells the mesher reads (a flowing liquid's extra
// horizontal neighbours are read from the chunk data directly).
constexpr int kCls = 34;
constexpr int kClsCells = kCls * kCls * kCls; // 39,304
// Light of [-1, 32]^3, the region the mesher reads.
constexpr int kLt = 34;
constexpr int kLtCells = kLt * kLt * kLt; // 39,304
// The relight window [-15, 47)^3 as 62 x 62 rows of 62-bit words (bit = x + 15).
constexpr int kWin = 62;
constexpr int kWinRows = kWin * kWin; // 3,844
// Per-chunk bit planes (pass, sun, level-15 emitters, opaque full cubes, blank blocks) as 32-bit
// rows (bit = x, row = z + 32 y), plus one flag bit per row (the row holds an emitter of level
// 1..14), a summary word per y layer (kLayer* bits: which kinds of block the layer and its edge
// rows hold), then the chunk's block class ids, one byte per cell in the reference's cell order.
constexpr int kPlaneWords = 1024;
enum { kPlanePass = 0, kPlaneSun = 1, kPlaneT15 = 2, kPlaneOpaque = 3, kPlaneEmpty = 4 };
constexpr int kPlaneLowOff = 5 * kPlaneWords;             // words: per y layer the low-emitter row bits
constexpr int kPlaneLayerOff = kPlaneLowOff + 32;         // words: per y layer a summary word
constexpr int kPlaneClassOff = kPlaneLowOff + 64;         // words
constexpr int kPlaneBits = kPlaneClassOff;                // the bit planes alone
constexpr int kPlaneStride = kPlaneClassOff + 32768 / 4; // 53,504 bytes per chunk
// Layer summary bits: some block with a texture or custom mesh; some block that is not an opaque
// full cube; the same for the x = 0 column, the x = 31 column, the z = 0 row and the z = 31 row;
// some block with a custom mesh.
enum : uint32_t {
	kLayerContent = 1, kLayerOpen = 2, kLayerOpenX0 = 4, kLayerOpenX31 = 8, kLayerOpenZ0 = 16, kLayerOpenZ31 = 32,
	kLayerCustom = 64
};
// Quad records staged for dense emission (two words each): kQuadBuf in shared memory, then up to
// kSpillRecs more per CTA in a global scratch (the most quads a chunk can have is 3 x 33 x 2 x 1,024
// = 202,752; beyond the scratch the emission merges the planes again in windows).
constexpr int kQuadBuf = 4096;
constexpr uint32_t kSpillRecs = 1u << 17;

// One block class: a distinct property row of the registry (65,536 raw values map onto < 256).
struct DevClass {
	uint16_t tex[6];
	uint8_t flags;     // kF* below
	uint8_t light;     // light level
	uint8_t mesh_first;// first static face (static meshes)
	uint8_t mesh_meta; // kind | count_or_variant << 2
};
static_assert(sizeof(DevClass) == 16, "DevClass is 16 bytes");

enum : uint8_t {
	kFIndirect = 1,   // transparency != opaque (light passes, BFS may enter)
	kFDirect = 2,     // vertical pass or no solid collision (AO does not darken)
	kFVertical = 4,   // transparency == transparent
	kFOpaqueCube = 8, // six non-empty, non-transparent textures and no custom mesh
	                  // (kFIndirect and kFDirect are also bits 7 and 6 of the class id itself)
	kFEmpty = 16,     // six empty textures and no custom mesh
	kFTagShift = 5    // 2-bit id tag
};
enum : uint8_t { kTagOther = 0, kTagAir = 1, kTagSource = 2, kTagFlow = 3 };

struct DevTables {
	const uint8_t *class_of;  // [65536]
	const DevClass *classes;  // [256]
};

// Texture flags (one bit per texture id) and static custom-mesh faces.
__constant__ uint64_t c_tex_transparent;
__constant__ uint64_t c_tex_liquid;
__constant__ uint64_t c_tex_transpass;
__constant__ hc_mesh_face c_static_faces[HC_MAX_STATIC_FACES / 4];

// Per-face neighbour offsets: the face-front cell, and per corner {side 0, diagonal, side 1}
// (client/include/client/BlockMeshAlgo.hpp:74-108).
__constant__ int8_t c_front[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
__constant__ int8_t c_corner[6][4][3][3] = {
    {{{1, 0, -1}, {1, -1, -1}, {1, -1, 0}},
     {{1, 0, -1}, {1, 1, -1}, {1, 1, 0}},
     {{1, 0, 1}, {1, 1, 1}, {1, 1, 0}},
     {{1, 0, 1}, {1, -1, 1}, {1, -1, 0}}},
    {{{-1, 0, -1}, {-1, -1, -1}, {-1, -1, 0}},
     {{-1, 0, 1}, {-1, -1, 1}, {-1, -1, 0}},
     {{-1, 0, 1}, {-1, 1, 1}, {-1, 1, 0}},
     {{-1, 0, -1}, {-1, 1, -1}, {-1, 1, 0}}},
    {{{0, 1, -1}, {-1, 1, -1}, {-1, 1, 0}},
     {{0, 1, 1}, {-1, 1, 1}, {-1, 1, 0}},
     {{0, 1, 1}, {1, 1, 1}, {1, 1, 0}},
     {{0, 1, -1}, {1, 1, -1}, {1, 1, 0}}},
    {{{0, -1, -1}, {-1, -1, -1}, {-1, -1, 0}},
     {{0, -1, -1}, {1, -1, -1}, {1, -1, 0}},
     {{0, -1, 1}, {1, -1, 1}, {1, -1, 0}},
     {{0, -1, 1}, {-1, -1, 1}, {-1, -1, 0}}},
    {{{0, -1, 1}, {-1, -1, 1}, {-1, 0, 1}},
     {{0, -1, 1}, {1, -1, 1}, {1, 0, 1}},
     {{0, 1, 1}, {1, 1, 1}, {1, 0, 1}},
     {{0, 1, 1}, {-1, 1, 1}, {-1, 0, 1}}},
    {{{0, -1, -1}, {-1, -1, -1}, {-1, 0, -1}},
     {{0, 1, -1}, {-1, 1, -1}, {-1, 0, -1}},
     {{0, 1, -1}, {1, 1, -1}, {1, 0, -1}},
     {{0, -1, -1}, {1, -1, -1}, {1, 0, -1}}}};

// Shared memory of one chunk CTA (about 215 KB: one CTA per SM).
constexpr int kRowWords = (kWinRows + 31) / 32;
struct Relight {
	uint64_t pass[kWinRows];   // blocks light may enter
	ulonglong2 lit[kWinRows];  // current level set: .x sun, .y torch
	uint32_t low_rows[kRowWords]; // rows holding emitters of level 1..14
	uint32_t changed[2][kRowWords]; // rows that changed at the last two levels
};
struct Smem {
	DevClass classes[256];
	uint8_t cflags[256]; // classes[c].flags, packed (fewer bank conflicts when lanes look up many classes)
	uint32_t cmesh[8];   // the classes with a custom mesh, as a 256-bit set
	const uint16_t *blk[27];
	const int8_t *hgt[27];
	const uint32_t *pln[27]; // per-chunk bit planes, or null (then the window is seeded from blocks)
	const uint32_t *lvl[27]; // per-chunk level planes of the batch light pass, or null (then relight the window)
	const uint32_t *edg[27]; // ... and their x = 0 / x = 31 edge bits
	uint32_t lfl[27][2];     // ... and their uniform-plane bits per channel (LightPass::flags)
	alignas(16) uint16_t cell[kClsCells + 8]; // per cell of [-1, 32]^3: light (low byte), class id (high byte)
	union {
		Relight rl;
		uint32_t masks[kPlanes][32][4]; // per plane row: visible, equal-right, equal-below, transparent pass
	} u;
	union {
		struct {
			uint64_t oc[kCls * kCls]; // x-row bits (bit = x + 1) of opaque full cubes, row = (z+1) + 34 (y+1)
			uint64_t em[kCls * kCls]; // ... of blocks with no texture and no custom mesh
		} pl;
		uint2 quads[kQuadBuf]; // staged quad records
	} aux;
	uint32_t seg_cnt[2][kSegments + 1];
	uint32_t seg_base[3][kSegments + 1]; // per stream and all-stream exclusive prefix
	uint32_t warp_sum[3][kWarps];
	uint32_t aabb[2][kMaxMeshesPerStream][6];
	uint32_t trig[2][kMaxMeshesPerStream];
	uint32_t misc[16];
	uint2 *spill;       // this CTA's quad records past kQuadBuf (global scratch), or null
	uint32_t spill_cap; // records it holds
	uint8_t plane_owner[kPlanes]; // cluster form, in CTA 0: the CTA that took each face plane
	uint8_t mine[kPlanes];        // the face planes this CTA took, in the order it took them
	uint8_t order[kPlanes];       // the face planes by falling face count: the order they are taken in
	uint8_t row_of[kWarps][32];   // per warp, key pass: the row whose faces start at each lane of a batch
	// face planes keyed in two halves (the heaviest): the visible and complex words of the row above
	// the second half, the second half's first row, and how many halves are done
	uint32_t split_side[kMaxSplit][kMaxParts][2]; // part q >= 1: visible and complex words of its first row - 1
	uint32_t split_done[kMaxSplit];
	uint8_t split_rows[kMaxSplit][kMaxParts + 1]; // part q keys rows [rows[q], rows[q + 1])
	uint8_t split_first[kMaxSplit + 1];           // claim index of each split plane's first part
	uint32_t lone_planes[(kPlanes + 31) / 32];    // planes all of whose faces are lone (emitted from their masks)
	int8_t lvl_slot[32];  // per light-level plane of the chunk (channel * 15 + level - 1): its copy in the staging scratch, or -1
	int8_t lvl_plane[16]; // ... and per copy, its plane
};

static_assert(offsetof(Smem, u) % 16 == 0, "plane mask rows are written as 16-byte words");

__device__ __forceinline__ int cls_index(int x, int y, int z) { return ((y + 1) * kCls + (z + 1)) * kCls + (x + 1); }
__device__ __forceinline__ int lt_index(int x, int y, int z) { return ((y + 1) * kLt + (z + 1)) * kLt + (x + 1); }

// Neighbour chunk index of a cell in [-32, 64)^3 (common/include/common/Position.hpp:138-145).
__device__ __forceinline__ int nb_index(int x, int y, int z) {
	int cx = x < 0 ? 1 : (x >= kChunk ? 0 : 2);
	int cy = y < 0 ? 1 : (y >= kChunk ? 0 : 2);
	int cz = z < 0 ? 1 : (z >= kChunk ? 0 : 2);
	return cx * 9 + cy * 3 + cz;
}
__device__ __forceinline__ uint16_t raw_at(const Smem &S, int x, int y, int z) {
	return S.blk[nb_index(x, y, z)][(x & 31) + ((y & 31) * kChunk + (z & 31)) * kChunk];
}
// Class id of a cell from the chunk planes (S.pln set for all 27 chunks).
__device__ __forceinline__ uint8_t class_byte(const Smem &S, int x, int y, int z) {
	const uint8_t *c = reinterpret_cast<const uint8_t *>(S.pln[nb_index(x, y, z)] + kPlaneClassOff);
	return __ldg(c + (x & 31) + ((y & 31) * kChunk + (z & 31)) * kChunk);
}
// Chunk::GetSunlight: unsigned local y >= the int8 height converted to unsigned (Chunk.hpp:74-76).
__device__ __forceinline__ bool sunlit(const Smem &S, int x, int y, int z) {
	int8_t h = S.hgt[nb_index(x, y, z)][(x & 31) + (z & 31) * kChunk];
	return (uint32_t)(y & 31) >= (uint32_t)(int32_t)h;
}

__device__ __forceinline__ bool tex_transparent(uint16_t t) { return (c_tex_transparent >> (t & 63u)) & 1u; }
__device__ __forceinline__ bool tex_liquid(uint16_t t) { return (c_tex_liquid >> (t & 63u)) & 1u; }
__device__ __forceinline__ bool tex_transpass(uint16_t t) { return (c_tex_transpass >> (t & 63u)) & 1u; }
__device__ __forceinline__ bool tex_empty(uint16_t t) { return (t & 0x1fffu) == 0; }

// BlockTexture::Show (texture/include/texture/BlockTexture.hpp:68-76).
__device__ __forceinline__ bool show(uint16_t a, uint16_t b) {
	if (tex_empty(a) || a == b)
		return false;
	const bool ta = tex_transparent(a), tb = tex_transparent(b);
	if (!ta && !tb)
		return false;
	if (tex_liquid(a) && !tex_empty(b))
		return false;
	return !ta || tb || tex_liquid(b);
}

__device__ __forceinline__ uint8_t class_at(const Smem &S, int x, int y, int z) { return S.cell[cls_index(x, y, z)] >> 8; }
// Class ids carry the two light-pass flags: bit 7 = light may pass (kFIndirect), bit 6 = does not
// darken ambient occlusion (kFDirect).
__device__ __forceinline__ bool id_indirect(uint32_t c) { return (c >> 7) & 1u; }
__device__ __forceinline__ bool id_direct(uint32_t c) { return (c >> 6) & 1u; }
__device__ __forceinline__ uint8_t tag_of(const DevClass &k) { return k.flags >> kFTagShift; }

// Dynamic face textures of a flowing liquid at (x, y, z) in [-1, 32]^3.
__device__ void flow_mesh_at(const Smem &S, int x, int y, int z, uint8_t variant, hc_mesh_face *faces, uint32_t *count,
                             uint16_t tex6[6]) {
	const int kF[8][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
	uint16_t nei[8];
#pragma unroll
	for (int i = 0; i < 8; ++i)
		nei[i] = raw_at(S, x + kF[i][0], y, z + kF[i][1]);
	hc_flow_mesh_impl(nei, variant, faces, count, tex6);
}

// Face texture of the block at (x, y, z), honouring flowing-liquid dynamic textures
// (BlockMeshAlgo.hpp:322-326).
__device__ __forceinline__ uint16_t get_tex(const Smem &S, int x, int y, int z, int face) {
	const DevClass &k = S.classes[class_at(S, x, y, z)];
	if (tag_of(k) == kTagFlow) {
		uint16_t t6[6];
		uint32_t n;
		flow_mesh_at(S, x, y, z, (uint8_t)(k.mesh_meta >> 2), nullptr, &n, t6);
		return t6[face];
	}
	return k.tex[face];
}

// Swizzle YZX (client/include/client/BlockAlgo.hpp:30-41, 70-81): plane axes (U, V) are (y, z) for
// x slices, (z, x) for y slices and (y, x) for z slices.
__device__ __forceinline__ void to_xyz(int axis, int a, int u, int v, int &x, int &y, int &z) {
	if (axis == 0)
		x = a, y = u, z = v;
	else if (axis == 1)
		x = v, y = a, z = u;
	else
		x = v, y = u, z = a;
}

// Light4 of a face (BlockMeshAlgo.hpp:48-163): per corner a 2-bit AO and smoothed sun / torch
// light in 0..60. Packed as sun bytes, torch bytes and the AO byte.
struct Light4 {
	uint32_t sun, torch, ao;
};


// Index offsets of the same neighbours in the 34^3 class and light arrays (x + 34 z + 34^2 y).
__host__ __device__ constexpr int cell_offset(int dx, int dy, int dz) { return dx + kCls * dz + kCls * kCls * dy; }
#define HC_O(a, b, c) cell_offset(a, b, c)
__constant__ int16_t c_front_off[6] = {HC_O(1, 0, 0), HC_O(-1, 0, 0), HC_O(0, 1, 0), HC_O(0, -1, 0), HC_O(0, 0, 1), HC_O(0, 0, -1)};
// The eight cells around the face-front cell in the face's plane, in the cyclic order in which
// corner v of BlockMeshAlgo.hpp's light4_init (tables at 74-108) reads sides ring[2v] and
// ring[2v + 2] (mod 8) and the corner ring[2v + 1]; each cell is loaded once per face.
__constant__ int16_t c_ring_off[6][8] = {
    {HC_O(1, -1, 0), HC_O(1, -1, -1), HC_O(1, 0, -1), HC_O(1, 1, -1), HC_O(1, 1, 0), HC_O(1, 1, 1), HC_O(1, 0, 1), HC_O(1, -1, 1)},
    {HC_O(-1, 0, -1), HC_O(-1, -1, -1), HC_O(-1, -1, 0), HC_O(-1, -1, 1), HC_O(-1, 0, 1), HC_O(-1, 1, 1), HC_O(-1, 1, 0),
     HC_O(-1, 1, -1)},
    {HC_O(0, 1, -1), HC_O(-1, 1, -1), HC_O(-1, 1, 0), HC_O(-1, 1, 1), HC_O(0, 1, 1), HC_O(1, 1, 1), HC_O(1, 1, 0), HC_O(1, 1, -1)},
    {HC_O(-1, -1, 0), HC_O(-1, -1, -1), HC_O(0, -1, -1), HC_O(1, -1, -1), HC_O(1, -1, 0), HC_O(1, -1, 1), HC_O(0, -1, 1),
     HC_O(-1, -1, 1)},
    {HC_O(-1, 0, 1), HC_O(-1, -1, 1), HC_O(0, -1, 1), HC_O(1, -1, 1), HC_O(1, 0, 1), HC_O(1, 1, 1), HC_O(0, 1, 1), HC_O(-1, 1, 1)},
    {HC_O(0, -1, -1), HC_O(-1, -1, -1), HC_O(-1, 0, -1), HC_O(-1, 1, -1), HC_O(0, 1, -1), HC_O(1, 1, -1), HC_O(1, 0, -1),
     HC_O(1, -1, -1)}};
#undef HC_O

// A cell's sun and torch levels side by side, sun in bits 0-7 and torch in bits 16-23, so that one
// addition sums both channels (four 4-bit levels times four stay below 256).
__device__ __forceinline__ uint32_t light_pair(uint32_t cell) { return (cell & 0x0fu) | ((cell & 0xf0u) << 12); }

// AO of one corner by the direct-pass bits of its side, corner and other side cell and of the
// face-front cell (index bits 0-3): 0 when both sides are blocked or the corner and the front are,
// else 3 minus the blocked cells, at least 0 (BlockMeshAlgo.hpp:127-131). Two bits per index.
constexpr uint32_t kAoTable = 0xe9849040u;

__device__ Light4 light4(const Smem &S, int face, int x, int y, int z) {
	const int base = cls_index(x, y, z);
	const uint32_t cf = S.cell[base + c_front_off[face]];
	const uint32_t pf = light_pair(cf);
	const uint32_t dp3 = (cf >> 11) & 8u; // the front cell's direct pass (class bit 6) as index bit 3
	uint32_t ring[8];
#pragma unroll
	for (int i = 0; i < 8; ++i)
		ring[i] = S.cell[base + c_ring_off[face][i]];
	uint32_t ipm = 0, dpm = 0; // bit i: ring cell i passes light indirectly (class bit 7) / directly (bit 6)
#pragma unroll
	for (int i = 0; i < 8; ++i) {
		ipm |= ((ring[i] >> 15) & 1u) << i;
		dpm |= ((ring[i] >> 14) & 1u) << i;
	}
	ipm |= ipm << 8, dpm |= dpm << 8; // so that the three cells of corner 3 (6, 7, 0) are consecutive
	Light4 r{0, 0, 0};
#pragma unroll
	for (int v = 0; v < 4; ++v) { // side, corner, side: ring cells 2v, 2v + 1, 2v + 2 (mod 8)
		const uint32_t d3 = (dpm >> (2 * v)) & 7u, i3 = (ipm >> (2 * v)) & 7u;
		const uint32_t ao = (kAoTable >> (2 * (d3 | dp3))) & 3u;
		// the front cell, plus every light-passing side or corner cell when a side passes light
		const uint32_t m = (i3 & 5u) ? i3 : 0u;
		const uint32_t sum = (pf + ((m & 1u) ? light_pair(ring[2 * v]) : 0u) + ((m & 2u) ? light_pair(ring[2 * v + 1]) : 0u) +
		                      ((m & 4u) ? light_pair(ring[(2 * v + 2) & 7]) : 0u))
		                     << 2;
		const uint32_t counter = 1u + (uint32_t)__popc(m);
		// (sum << 2) / counter in both halves: a shift for 1, 2 and 4; for 3 the multiply-high by
		// 171 / 512, exact for every value up to 240 (Granlund and Montgomery, "Division by invariant
		// integers using multiplication", 1994), the sun product staying below bit 16. A plain
		// integer division here would cost eight software divisions per face.
		const uint32_t pr = sum * 171u;
		const uint32_t q = counter == 3 ? (((pr >> 9) & 0x7fu) | (((pr >> 25) & 0x7fu) << 16))
		                                : ((sum >> (counter >> 1)) & 0x00ff00ffu);
		r.ao |= ao << (2 * v);
		r.sun |= (q & 0xffu) << (8 * v);
		r.torch |= (q >> 16) << (8 * v);
	}
	return r;
}

__device__ __forceinline__ uint32_t l4_get(uint32_t packed, int i) { return (packed >> (8 * i)) & 0xffu; }
__device__ __forceinline__ uint32_t ao_get(uint32_t ao, int i) { return (ao >> (2 * i)) & 3u; }

// Light4::GetFlip (BlockMeshAlgo.hpp:38-43).
__device__ __forceinline__ bool flip_of(const Light4 &l) {
	int a = (int)((ao_get(l.ao, 0) + 1) * (l4_get(l.sun, 0) + 1)) - (int)((ao_get(l.ao, 2) + 1) * (l4_get(l.sun, 2) + 1));
	int b = (int)((ao_get(l.ao, 1) + 1) * (l4_get(l.sun, 1) + 1)) - (int)((ao_get(l.ao, 3) + 1) * (l4_get(l.sun, 3) + 1));
	return abs(a) < abs(b);
}

// Packed vertex (client/include/client/BlockVertex.hpp:13-17).
__device__ __forceinline__ uint2 pack_vertex(uint32_t x, uint32_t y, uint32_t z, uint32_t axis, uint32_t face, uint32_t ao,
                                             uint32_t sun, uint32_t torch, uint16_t texture) {
	uint32_t id = texture & 0x1fffu, trans = (uint32_t)texture >> 13;
	return make_uint2(x | (y << 10u) | (z << 20u) | (axis << 30u),
	                  (id - 1u) | (trans << 10u) | (face << 13u) | (ao << 16u) | (sun << 18u) | (torch << 24u));
}

} // namespace hc
