// CPU oracle: a plain restatement of HyperCraft's chunk relight + mesh call.
//
// TEST INFRASTRUCTURE. Only tests/, the smoke check and bench.py's CPU-baseline leg load this
// library, and only as the checker or the timed CPU baseline; the product never links it.
//
// What it restates (paths inside the reference project):
//   kMesh runner glue ........ client/src/ChunkMeshTask.cpp:41-122 (seed 49-87, BFS 89-111, mesh 113-122)
//   window index ............. client/src/ChunkMeshTask.cpp:10-12
//   light BFS ................ client/include/client/BlockLightAlgo.hpp:24-73 (Border = 14,
//                              bound [-1,33)^3 from client/include/client/ChunkMeshTask.inl:53-56)
//   mesher ................... client/include/client/BlockMeshAlgo.hpp:17-521
//   loop/swizzle order ....... client/include/client/BlockAlgo.hpp:20-95 (YZX)
//   vertex packing ........... client/include/client/BlockVertex.hpp:8-25
//   neighbour addressing ..... client/include/client/Chunk.hpp:57-82, common/include/common/Position.hpp:98-152
//   AABB merge ............... dep/AABB.hpp:9-59
// Parity: this restatement is pinned against the reference's own templates compiled from source
// (oracle/ref_harness.cpp), and through committed golden fixtures where the reference is absent.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <deque>
#include <thread>
#include <vector>

#include "../hypercraft_gb300/csrc/hc_registry.h"
#include "hc_flat.h"

namespace {

constexpr int kSize = 32;
constexpr int kExt = kSize + 30; // the 62^3 light window [-15, 47)^3

const hc_registry &registry() {
	static hc_registry *r = [] {
		hc_registry *p = (hc_registry *)std::malloc(sizeof(hc_registry));
		hc_registry_build(p);
		return p;
	}();
	return *r;
}

inline const hc_block_props &props(uint16_t raw) { return registry().props[raw]; }
inline bool indirect_pass(uint16_t raw) { return props(raw).transparency != HC_OPAQUE; }
inline bool vertical_pass(uint16_t raw) { return props(raw).transparency == HC_TRANSPARENT; }

// Position.hpp:138-145: neighbour chunk index (centre = 26).
inline int neighbour_index(int x, int y, int z) {
	static const int kLookUp[3] = {1, 2, 0};
	int cx = x < 0 ? -1 : (x >= kSize ? 1 : 0), cy = y < 0 ? -1 : (y >= kSize ? 1 : 0),
	    cz = z < 0 ? -1 : (z >= kSize ? 1 : 0);
	return kLookUp[cx + 1] * 9 + kLookUp[cy + 1] * 3 + kLookUp[cz + 1];
}

struct World27 {
	const uint16_t *const *blocks;
	const int8_t *const *heights;
	uint16_t block(int x, int y, int z) const {
		int n = neighbour_index(x, y, z);
		int lx = (x + kSize) % kSize, ly = (y + kSize) % kSize, lz = (z + kSize) % kSize;
		return blocks[n][lx + (ly * kSize + lz) * kSize];
	}
	// Chunk::GetSunlight compares the unsigned local y against the int8 height converted the
	// same way (Chunk.hpp:74-76), so a negative height never lights.
	bool sunlight(int x, int y, int z) const {
		int n = neighbour_index(x, y, z);
		int lx = (x + kSize) % kSize, ly = (y + kSize) % kSize, lz = (z + kSize) % kSize;
		return (uint32_t)ly >= (uint32_t)(int32_t)heights[n][lx + lz * kSize];
	}
};

inline int ext_index(int x, int y, int z) { return x + 15 + ((z + 15) + (y + 15) * kExt) * kExt; }

// BlockLightAlgo.hpp:25-42 with bound [-1,33)^3 and Border 14.
inline bool in_bound_bordered(int x, int y, int z) {
	return -15 <= x && x < 47 && -15 <= y && y < 47 && -15 <= z && z < 47;
}
inline uint32_t axis_dist(int v) { return v < -1 ? (uint32_t)(-1 - v) : (v >= 33 ? (uint32_t)(v - 33) : 0u); }
inline bool border_interfere(int x, int y, int z, uint32_t lvl) {
	return lvl > axis_dist(x) + axis_dist(y) + axis_dist(z);
}

struct Entry {
	int8_t x, y, z;
	uint8_t lvl;
};

// One light channel of the window: nibble 0 = sun, 1 = torch.
void propagate(std::deque<Entry> &q, const World27 &w, uint8_t *light, int nibble) {
	const int shift = nibble * 4;
	while (!q.empty()) {
		Entry e = q.front();
		q.pop_front();
		if (e.lvl <= 1u)
			continue;
		uint8_t lvl = (uint8_t)(e.lvl - 1);
		for (int f = 0; f < 6; ++f) {
			int p[3] = {e.x, e.y, e.z};
			p[f >> 1] += 1 - ((f & 1) << 1);
			if (!in_bound_bordered(p[0], p[1], p[2]))
				continue;
			if (!border_interfere(p[0], p[1], p[2], lvl))
				continue;
			uint8_t &cell = light[ext_index(p[0], p[1], p[2])];
			if (lvl > ((cell >> shift) & 15u) && indirect_pass(w.block(p[0], p[1], p[2]))) {
				cell = (uint8_t)((cell & ~(15u << shift)) | (lvl << shift));
				if (lvl > 1)
					q.push_back({(int8_t)p[0], (int8_t)p[1], (int8_t)p[2], lvl});
			}
		}
	}
}

void relight_window(const World27 &w, uint8_t *light) {
	std::deque<Entry> sun_q, torch_q;
	for (int y = -15; y < kSize + 15; ++y)
		for (int z = -15; z < kSize + 15; ++z)
			for (int x = -15; x < kSize + 15; ++x) {
				uint8_t torch = props(w.block(x, y, z)).light_level;
				uint8_t sun = w.sunlight(x, y, z) ? 15 : 0;
				light[ext_index(x, y, z)] = (uint8_t)((torch << 4) | sun);
				if (border_interfere(x, y, z, torch))
					torch_q.push_back({(int8_t)x, (int8_t)y, (int8_t)z, torch});
			}
	const auto lit = [light](int x, int y, int z) { return (light[ext_index(x, y, z)] & 15u) == 15u; };
	for (int y = -15; y < kSize + 15; ++y)
		for (int z = -15; z < kSize + 15; ++z)
			for (int x = -15; x < kSize + 15; ++x) {
				uint8_t sun = light[ext_index(x, y, z)] & 15u;
				if (!border_interfere(x, y, z, sun))
					continue;
				// a fully lit cell whose six neighbours are fully lit (window edges count) adds nothing
				if ((x == -15 || lit(x - 1, y, z)) && (x == kSize + 14 || lit(x + 1, y, z)) &&
				    (z == -15 || lit(x, y, z - 1)) && (z == kSize + 14 || lit(x, y, z + 1)) &&
				    (y == -15 || lit(x, y - 1, z)) && (y == kSize + 14 || lit(x, y + 1, z)))
					continue;
				sun_q.push_back({(int8_t)x, (int8_t)y, (int8_t)z, sun});
			}
	propagate(sun_q, w, light, 0);
	propagate(torch_q, w, light, 1);
}

// ---------------------------------------------------------------- mesher (BlockMeshAlgo.hpp)

struct Light4 {
	uint8_t sun[4], torch[4];
	uint8_t ao; // 2 bits per corner
	bool operator==(const Light4 &r) const {
		return ao == r.ao && std::memcmp(sun, r.sun, 4) == 0 && std::memcmp(torch, r.torch, 4) == 0;
	}
	bool operator!=(const Light4 &r) const { return !(*this == r); }
	uint8_t get_ao(int i) const { return (ao >> (2 * i)) & 3u; }
	void set_ao(int i, uint8_t v) { ao = (uint8_t)((ao & ~(3u << (2 * i))) | (v << (2 * i))); }
	// BlockMeshAlgo.hpp:38-43
	bool flip() const {
		int a = (get_ao(0) + 1) * (sun[0] + 1) - (get_ao(2) + 1) * (sun[2] + 1);
		int b = (get_ao(1) + 1) * (sun[1] + 1) - (get_ao(3) + 1) * (sun[3] + 1);
		return std::abs(a) < std::abs(b);
	}
};

// Neighbour offsets per face and corner: {side 0, diagonal, side 1} (BlockMeshAlgo.hpp:74-108).
const int8_t kFront[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
const int8_t kCorner[6][4][3][3] = {
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

struct Mesh {
	std::vector<uint32_t> vertices; // two words per vertex
	std::vector<uint16_t> indices;
	uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0, 0, 0};
	bool transparent = false;
	uint32_t vertex_count() const { return (uint32_t)(vertices.size() / 2); }
	void merge(uint32_t x, uint32_t y, uint32_t z) {
		const uint32_t p[3] = {x, y, z};
		for (int k = 0; k < 3; ++k) {
			mn[k] = p[k] < mn[k] ? p[k] : mn[k];
			mx[k] = p[k] > mx[k] ? p[k] : mx[k];
		}
	}
	void vertex(uint32_t x, uint32_t y, uint32_t z, uint32_t axis, uint32_t face, uint32_t ao, uint32_t sun,
	            uint32_t torch, uint16_t texture) {
		uint32_t id = texture & 0x1fffu, trans = texture >> 13;
		vertices.push_back(x | (y << 10u) | (z << 20u) | (axis << 30u));
		vertices.push_back((id - 1u) | (trans << 10u) | (face << 13u) | (ao << 16u) | (sun << 18u) | (torch << 24u));
	}
};

struct Mesher {
	const World27 &w;
	const uint8_t *light; // the 62^3 window
	std::vector<Mesh> meshes;
	Mesh opaque, transparent;
	// dynamic textures over [-1, 32]^3 (the reference keys an unordered_map by position)
	std::vector<uint16_t> dyn_tex;
	std::vector<uint8_t> has_dyn;

	Mesher(const World27 &w_, const uint8_t *l) : w(w_), light(l), dyn_tex(34 * 34 * 34 * 6), has_dyn(34 * 34 * 34) {
		transparent.transparent = true;
	}
	static int dyn_index(int x, int y, int z) { return (x + 1) + ((y + 1) * 34 + (z + 1)) * 34; }
	uint8_t light_at(int x, int y, int z) const { return light[ext_index(x, y, z)]; }

	// BlockMeshAlgo.hpp:48-163
	void light4_init(Light4 &l4, int face, int x, int y, int z) const {
		const int fx = x + kFront[face][0], fy = y + kFront[face][1], fz = z + kFront[face][2];
		for (int v = 0; v < 4; ++v) {
			bool ip[3], dp[4];
			for (int b = 0; b < 3; ++b) {
				uint16_t blk = w.block(x + kCorner[face][v][b][0], y + kCorner[face][v][b][1], z + kCorner[face][v][b][2]);
				ip[b] = indirect_pass(blk);
				dp[b] = vertical_pass(blk) || props(blk).collision != HC_COLLISION_SOLID;
			}
			{
				uint16_t blk = w.block(fx, fy, fz);
				dp[3] = vertical_pass(blk) || props(blk).collision != HC_COLLISION_SOLID;
			}
			int blocked = !dp[0] + !dp[1] + !dp[2] + !dp[3];
			uint32_t ao = ((!dp[0] && !dp[2]) || (!dp[1] && !dp[3])) ? 0u : (uint32_t)(3 - blocked > 0 ? 3 - blocked : 0);
			l4.set_ao(v, (uint8_t)ao);
			uint32_t counter = 1;
			uint8_t l = light_at(fx, fy, fz);
			uint32_t sun = l & 15u, torch = l >> 4;
			if (ip[0] || ip[2]) {
				for (int b = 0; b < 3; ++b)
					if (ip[b]) {
						++counter;
						uint8_t lb =
						    light_at(x + kCorner[face][v][b][0], y + kCorner[face][v][b][1], z + kCorner[face][v][b][2]);
						sun += lb & 15u;
						torch += lb >> 4;
					}
			}
			l4.sun[v] = (uint8_t)((sun << 2u) / counter);
			l4.torch[v] = (uint8_t)((torch << 2u) / counter);
		}
	}

	// BlockMeshAlgo.hpp:165-196 (trilinear interpolation in 1/16 units, rounded up)
	static void interpolate(const Light4 &lo, const Light4 &hi, uint32_t du, uint32_t dv, uint32_t dw, uint8_t *ao,
	                        uint8_t *sun, uint8_t *torch) {
		const auto lerp = [](uint32_t a, uint32_t b, uint32_t t) { return a * (16u - t) + b * t; };
		const auto ceil_div = [](uint32_t a) { return a / 4096u + (a % 4096u ? 1u : 0u); };
		if (*ao == 4) {
			uint32_t s = lerp(lerp(lerp(lo.get_ao(0), lo.get_ao(1), du), lerp(lo.get_ao(3), lo.get_ao(2), du), dv),
			                  lerp(lerp(hi.get_ao(0), hi.get_ao(1), du), lerp(hi.get_ao(3), hi.get_ao(2), du), dv), dw);
			*ao = (uint8_t)ceil_div(s);
		}
		uint32_t s = lerp(lerp(lerp(lo.sun[0], lo.sun[1], du), lerp(lo.sun[3], lo.sun[2], du), dv),
		                  lerp(lerp(hi.sun[0], hi.sun[1], du), lerp(hi.sun[3], hi.sun[2], du), dv), dw);
		*sun = (uint8_t)ceil_div(s);
		uint32_t t = lerp(lerp(lerp(lo.torch[0], lo.torch[1], du), lerp(lo.torch[3], lo.torch[2], du), dv),
		                  lerp(lerp(hi.torch[0], hi.torch[1], du), lerp(hi.torch[3], hi.torch[2], du), dv), dw);
		*torch = (uint8_t)ceil_div(t);
	}

	// Start a new mesh of the stream when four more vertices would overflow uint16 indices
	// (BlockMeshAlgo.hpp:272-279, 396-403). The reference reads the base index *before* the split,
	// so the first quad of every continuation mesh indexes from 65532; *cur receives that value.
	Mesh &stream(bool trans_pass, uint16_t *cur) {
		Mesh &m = trans_pass ? transparent : opaque;
		*cur = (uint16_t)m.vertex_count();
		if (m.vertex_count() + 4 > 65535u) {
			bool t = m.transparent;
			meshes.push_back(std::move(m));
			m = Mesh{};
			m.transparent = t;
		}
		return m;
	}

	// BlockMeshAlgo.hpp:198-306
	void custom_meshes() {
		const hc_registry &r = registry();
		for (int y = -1; y <= kSize; ++y)
			for (int z = -1; z <= kSize; ++z)
				for (int x = -1; x <= kSize; ++x) {
					const bool inner = 0 <= x && x < kSize && 0 <= y && y < kSize && 0 <= z && z < kSize;
					const hc_block_props &p = props(w.block(x, y, z));
					if (p.mesh_kind == HC_MESH_NONE)
						continue;
					hc_mesh_face dyn[HC_MAX_MESH_FACES];
					const hc_mesh_face *faces = r.static_faces + p.mesh_first;
					uint32_t face_count = p.mesh_count;
					if (p.mesh_kind == HC_MESH_FLOW) {
						// fetch order of kLiquidFlowMesh (Liquid.hpp:291-300)
						static const int kFetch[8][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
						uint16_t nei[8];
						for (int i = 0; i < 8; ++i)
							nei[i] = w.block(x + kFetch[i][0], y, z + kFetch[i][1]);
						uint16_t tex6[6];
						hc_flow_mesh(nei, p.flow_variant, dyn, &face_count, tex6);
						int di = dyn_index(x, y, z);
						has_dyn[di] = 1;
						std::memcpy(&dyn_tex[di * 6], tex6, sizeof(tex6));
						faces = dyn;
					}
					if (!inner)
						continue;
					const uint32_t base[3] = {(uint32_t)x << 4, (uint32_t)y << 4, (uint32_t)z << 4};
					int cur_face = 255, cur_axis = 0, u_axis = 0, v_axis = 0;
					Light4 lo{}, hi{};
					for (uint32_t i = 0; i < face_count; ++i) {
						const hc_mesh_face &f = faces[i];
						if (f.light_face != cur_face) {
							cur_face = f.light_face;
							cur_axis = cur_face >> 1;
							u_axis = (cur_axis + 1) % 3;
							v_axis = (cur_axis + 2) % 3;
							if (cur_face & 1) {
								int t = u_axis;
								u_axis = v_axis;
								v_axis = t;
							}
							int op[3] = {x, y, z}, ne[3] = {x, y, z};
							op[cur_axis] -= 1 - ((cur_face & 1) << 1);
							ne[cur_axis] += 1 - ((cur_face & 1) << 1);
							light4_init(lo, cur_face, op[0], op[1], op[2]);
							if (indirect_pass(w.block(ne[0], ne[1], ne[2])))
								light4_init(hi, cur_face, x, y, z);
							else
								hi = lo;
						}
						uint16_t cur;
						Mesh &m = stream(hc_tex_use_transparent_pass(f.texture), &cur);
						for (int k = 0; k < 4; ++k) {
							const hc_mesh_vertex &v = f.v[k];
							m.merge(base[0] + v.pos[0], base[1] + v.pos[1], base[2] + v.pos[2]);
							uint32_t du = v.pos[u_axis], dv = v.pos[v_axis];
							uint32_t dw = v.pos[cur_axis] < 16 ? v.pos[cur_axis] : 16u;
							if (cur_face & 1)
								dw = 16u - dw;
							uint8_t ao = v.ao, sun, torch;
							interpolate(lo, hi, du, dv, dw, &ao, &sun, &torch);
							m.vertex(base[0] + v.pos[0], base[1] + v.pos[1], base[2] + v.pos[2], f.axis, f.render_face,
							         ao, sun, torch, f.texture);
						}
						const uint16_t idx[6] = {cur, (uint16_t)(cur + 1), (uint16_t)(cur + 2),
						                         cur, (uint16_t)(cur + 2), (uint16_t)(cur + 3)};
						m.indices.insert(m.indices.end(), idx, idx + 6);
					}
				}
	}

	uint16_t get_tex(int x, int y, int z, int face) const {
		if (x >= -1 && x <= kSize && y >= -1 && y <= kSize && z >= -1 && z <= kSize) {
			int di = dyn_index(x, y, z);
			if (has_dyn[di])
				return dyn_tex[di * 6 + face];
		}
		return props(w.block(x, y, z)).tex[face];
	}

	// BlockTexture::Show (texture/include/texture/BlockTexture.hpp:68-76)
	static bool show(uint16_t a, uint16_t b) {
		if ((a & 0x1fffu) == 0 || a == b)
			return false;
		if (!hc_tex_is_transparent(a) && !hc_tex_is_transparent(b))
			return false;
		if (hc_tex_is_liquid(a) && (b & 0x1fffu) != 0)
			return false;
		return !hc_tex_is_transparent(a) || hc_tex_is_transparent(b) || hc_tex_is_liquid(b);
	}

	// Swizzle YZX (BlockAlgo.hpp:30-41, 70-81): plane axes (U, V) per axis.
	static void to_xyz(int axis, int a, int u, int v, int out[3]) {
		if (axis == 0)
			out[0] = a, out[1] = u, out[2] = v;
		else if (axis == 1)
			out[0] = v, out[1] = a, out[2] = u;
		else
			out[0] = v, out[1] = u, out[2] = a;
	}

	// BlockMeshAlgo.hpp:308-482
	void regular_axis(int axis) {
		thread_local uint16_t tex_mask[2][1024]; // persists across slices like the reference's locals
		thread_local Light4 light_mask[2][1024];
		std::memset(tex_mask, 0, sizeof(tex_mask));
		const int u_axis = axis == 1 ? 2 : 1, v_axis = axis == 0 ? 2 : 0;
		const bool uv_cycle = (u_axis + 1) % 3 == v_axis;
		for (int xa = 0; xa <= kSize; ++xa) {
			uint8_t face_mask = 0;
			for (int u = 0, counter = 0; u < kSize; ++u)
				for (int v = 0; v < kSize; ++v, ++counter) {
					int p[3], n[3];
					to_xyz(axis, xa, u, v, p);
					n[0] = p[0], n[1] = p[1], n[2] = p[2];
					n[axis] -= 1;
					const int fa = axis << 1, fb = fa | 1;
					uint16_t ta = get_tex(n[0], n[1], n[2], fa), tb = get_tex(p[0], p[1], p[2], fb);
					if (xa != 0 && show(ta, tb)) {
						tex_mask[0][counter] = ta;
						light4_init(light_mask[0][counter], fa, n[0], n[1], n[2]);
						face_mask |= 1u;
					}
					if (xa != kSize && show(tb, ta)) {
						tex_mask[1][counter] = tb;
						light4_init(light_mask[1][counter], fb, p[0], p[1], p[2]);
						face_mask |= 2u;
					}
				}
			for (int inv = 0; inv < 2; ++inv) {
				if (!(face_mask & (1u << inv)))
					continue;
				uint16_t *tm = tex_mask[inv];
				Light4 *lm = light_mask[inv];
				for (int u = 0, counter = 0; u < kSize; ++u)
					for (int v = 0; v < kSize;) {
						const uint16_t qt = tm[counter];
						if (!(qt & 0x1fffu)) {
							++v, ++counter;
							continue;
						}
						const Light4 ql = lm[counter];
						int width = 1, height = 1;
						while (v + width < kSize && tm[counter + width] == qt && lm[counter + width] == ql)
							++width;
						for (; u + height < kSize; ++height) {
							bool ok = true;
							for (int k = 0; k < width && ok; ++k) {
								int idx = counter + k + height * kSize;
								ok = tm[idx] == qt && lm[idx] == ql;
							}
							if (!ok)
								break;
						}
						int o[3], du[3] = {0, 0, 0}, dv[3] = {0, 0, 0};
						to_xyz(axis, xa, u, v, o);
						int hv[3], wv[3];
						to_xyz(axis, 0, height, 0, hv);
						to_xyz(axis, 0, 0, width, wv);
						if (inv ^ (uv_cycle ? 1 : 0)) {
							std::memcpy(du, hv, sizeof(du));
							std::memcpy(dv, wv, sizeof(dv));
						} else {
							std::memcpy(du, wv, sizeof(du));
							std::memcpy(dv, hv, sizeof(dv));
						}
						uint16_t cur;
						Mesh &m = stream(hc_tex_use_transparent_pass(qt), &cur);
						m.merge((uint32_t)o[0] << 4, (uint32_t)o[1] << 4, (uint32_t)o[2] << 4);
						m.merge((uint32_t)(o[0] + du[0] + dv[0]) << 4, (uint32_t)(o[1] + du[1] + dv[1]) << 4,
						        (uint32_t)(o[2] + du[2] + dv[2]) << 4);
						const uint32_t face = (uint32_t)((axis << 1) | inv);
						const int corners[4][3] = {{o[0], o[1], o[2]},
						                           {o[0] + du[0], o[1] + du[1], o[2] + du[2]},
						                           {o[0] + du[0] + dv[0], o[1] + du[1] + dv[1], o[2] + du[2] + dv[2]},
						                           {o[0] + dv[0], o[1] + dv[1], o[2] + dv[2]}};
						for (int k = 0; k < 4; ++k)
							m.vertex((uint32_t)corners[k][0] << 4, (uint32_t)corners[k][1] << 4,
							         (uint32_t)corners[k][2] << 4, (uint32_t)axis, face, ql.get_ao(k), ql.sun[k],
							         ql.torch[k], qt);
						if (ql.flip()) {
							const uint16_t idx[6] = {cur, (uint16_t)(cur + 1), (uint16_t)(cur + 2),
							                         cur, (uint16_t)(cur + 2), (uint16_t)(cur + 3)};
							m.indices.insert(m.indices.end(), idx, idx + 6);
						} else {
							const uint16_t idx[6] = {(uint16_t)(cur + 1), (uint16_t)(cur + 2), (uint16_t)(cur + 3),
							                         cur, (uint16_t)(cur + 1), (uint16_t)(cur + 3)};
							m.indices.insert(m.indices.end(), idx, idx + 6);
						}
						for (int a = 0; a < height; ++a)
							std::memset(tm + counter + a * kSize, 0, sizeof(uint16_t) * width);
						v += width;
						counter += width;
					}
			}
		}
	}

	void generate() {
		custom_meshes();
		regular_axis(0);
		regular_axis(1);
		regular_axis(2);
		if (opaque.vertex_count())
			meshes.push_back(std::move(opaque));
		if (transparent.vertex_count())
			meshes.push_back(std::move(transparent));
	}
};

int write_flat(const std::vector<Mesh> &meshes, hc_flat_meshes *out) {
	uint32_t nv = 0, ni = 0;
	for (const auto &m : meshes)
		nv += m.vertex_count(), ni += (uint32_t)m.indices.size();
	out->mesh_count = (uint32_t)meshes.size();
	out->vertex_count = nv;
	out->index_count = ni;
	if (meshes.size() > out->mesh_cap || nv > out->vertex_cap || ni > out->index_cap)
		return 1;
	uint32_t vo = 0, io = 0;
	for (size_t i = 0; i < meshes.size(); ++i) {
		const Mesh &m = meshes[i];
		uint32_t *wds = out->meshes + i * HC_FLAT_MESH_WORDS;
		wds[0] = m.vertex_count();
		wds[1] = (uint32_t)m.indices.size();
		for (int k = 0; k < 3; ++k)
			wds[2 + k] = m.mn[k], wds[5 + k] = m.mx[k];
		wds[8] = m.transparent ? 1u : 0u;
		std::memcpy(out->vertices + 2 * vo, m.vertices.data(), m.vertices.size() * sizeof(uint32_t));
		std::memcpy(out->indices + io, m.indices.data(), m.indices.size() * sizeof(uint16_t));
		vo += m.vertex_count();
		io += (uint32_t)m.indices.size();
	}
	return 0;
}

thread_local std::vector<uint8_t> t_window;

} // namespace

extern "C" {

// Relights one chunk's 62^3 window (index x+15 + ((z+15) + (y+15)*62)*62; sun low nibble).
void hco_relight_window(const uint16_t *const *blocks, const int8_t *const *heights, uint8_t *light62) {
	World27 w{blocks, heights};
	relight_window(w, light62);
}

// Relight + mesh of the centre chunk (neighbour index 26) in reference order.
int hco_mesh_chunk(const uint16_t *const *blocks, const int8_t *const *heights, hc_flat_meshes *out) {
	World27 w{blocks, heights};
	t_window.resize((size_t)kExt * kExt * kExt);
	relight_window(w, t_window.data());
	Mesher m(w, t_window.data());
	m.generate();
	return write_flat(m.meshes, out);
}

// Mesh only, with a caller-provided 62^3 light window.
int hco_mesh_chunk_lit(const uint16_t *const *blocks, const int8_t *const *heights, const uint8_t *light62,
                       hc_flat_meshes *out) {
	World27 w{blocks, heights};
	Mesher m(w, light62);
	m.generate();
	return write_flat(m.meshes, out);
}

// Dumps the registry restatement in the layout of hcref_dump_registry's per-raw arrays.
void hco_dump_registry(uint16_t *tex6, uint8_t *transparency, uint8_t *light, uint8_t *collision, uint8_t *mesh_kind,
                       uint8_t *mesh_first, uint8_t *mesh_count, uint8_t *static_faces /*256*24*/,
                       uint32_t *static_face_count) {
	const hc_registry &r = registry();
	for (uint32_t raw = 0; raw < 65536u; ++raw) {
		const hc_block_props &p = r.props[raw];
		std::memcpy(tex6 + raw * 6, p.tex, 12);
		transparency[raw] = p.transparency;
		light[raw] = p.light_level;
		collision[raw] = p.collision;
		mesh_kind[raw] = p.mesh_kind;
		mesh_first[raw] = p.mesh_first;
		mesh_count[raw] = p.mesh_count;
	}
	std::memcpy(static_faces, r.static_faces, sizeof(hc_mesh_face) * r.static_face_count);
	*static_face_count = r.static_face_count;
}

void hco_flow_mesh(const uint16_t *nei8, uint8_t variant, uint8_t *faces_out, uint32_t *face_count, uint16_t *tex6) {
	hc_flow_mesh(nei8, variant, (hc_mesh_face *)faces_out, face_count, tex6);
}

// ChunkShouldRemesh (client/include/client/ChunkMeshTask.inl:9-15).
int hco_chunk_should_remesh(int x, int y, int z) { return border_interfere(x, y, z, 15) ? 1 : 0; }

// Meshes n chunks of a resident world (chunk c at blocks + c*32768, heights + c*1024; nbr holds 27
// chunk indices per item) on `threads` threads, each with its own window and mesher state, the way
// the reference's worker threads each own a runner. Returns the total quad count.
uint64_t hco_mesh_many(const uint16_t *blocks, const int8_t *heights, const int32_t *nbr, uint32_t n, int threads,
                       uint64_t *meshes_out) {
	std::atomic<uint32_t> next{0};
	std::atomic<uint64_t> quads{0}, meshes{0};
	const auto work = [&] {
		std::vector<uint8_t> window((size_t)kExt * kExt * kExt);
		const uint16_t *b27[27];
		const int8_t *h27[27];
		for (uint32_t i; (i = next.fetch_add(1)) < n;) {
			for (int k = 0; k < 27; ++k) {
				b27[k] = blocks + (size_t)nbr[(size_t)i * 27 + k] * 32768;
				h27[k] = heights + (size_t)nbr[(size_t)i * 27 + k] * 1024;
			}
			World27 w{b27, h27};
			relight_window(w, window.data());
			Mesher m(w, window.data());
			m.generate();
			uint64_t q = 0;
			for (const auto &mesh : m.meshes)
				q += mesh.vertex_count() / 4;
			quads += q;
			meshes += m.meshes.size();
		}
	};
	std::vector<std::thread> ts;
	for (int t = 1; t < threads; ++t)
		ts.emplace_back(work);
	work();
	for (auto &t : ts)
		t.join();
	if (meshes_out)
		*meshes_out = meshes;
	return quads;
}

} // extern "C"
