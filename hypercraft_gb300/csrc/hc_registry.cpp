// Restatement of HyperCraft's block registry as one property row per raw uint16 block value.
//
// Sources restated here (all paths inside the reference project):
//   texture flags ........ texture/internal/generated/block_texture_transparency.inl:1-3
//   variant/transform .... block/generator/Block.cpp.in:9-15, block/block/public/Trait.hpp:24-64
//   per-id properties .... block/block/*.hpp (air.hpp ... glowstone.hpp)
//   rotation of logs ..... block/include/block/BlockProperty.hpp:30-75, block/block/log.hpp:26-35
//   cross meshes ......... block/block/public/CrossMesh.hpp:7-52
//   inner-surface meshes . block/block/public/InnerSurfaceMesh.hpp:7-43
//   cactus ............... block/block/cactus.hpp:4-48
//   liquid flow mesh ..... block/block/public/Liquid.hpp:151-155 (heights), 156-282 (faces), 284-302 (kLiquidFlowMesh), Water.hpp:5-14
#include "hc_registry.h"
#include "hc_flow.h"

#include <initializer_list>
#include <string.h>

namespace {

// Texture flag sets, one bit per texture id.
constexpr uint64_t bits(std::initializer_list<int> ids) {
	uint64_t m = 0;
	for (int i : ids)
		m |= 1ull << i;
	return m;
}
constexpr uint64_t kTransparentTex = bits({0, 4, 7, 10, 13, 18, 21, 23, 24, 28, 32, 36, 40, 44, 45, 46, 47, 48, 49, 50, 51});
constexpr uint64_t kTransPassTex = bits({4, 7, 10, 13, 21, 23, 24, 28, 32, 36, 40});
constexpr uint64_t kLiquidTex = bits({23});

inline uint16_t tex(uint16_t id, uint8_t trans = 0) { return (uint16_t)((trans << 13) | id); }
inline uint16_t tex_id(uint16_t t) { return t & 0x1fff; }
inline uint8_t tex_trans(uint16_t t) { return (uint8_t)(t >> 13); }
inline uint16_t rot_cw(uint16_t t) { return tex(tex_id(t), tex_trans(t) ^ (HC_TRANS_SWAP_UV | HC_TRANS_NEG_U)); }
inline uint16_t rot_ccw(uint16_t t) { return tex(tex_id(t), tex_trans(t) ^ (HC_TRANS_SWAP_UV | HC_TRANS_NEG_V)); }
inline uint16_t swap_uv(uint16_t t) { return tex(tex_id(t), tex_trans(t) ^ HC_TRANS_SWAP_UV); }

int countr_zero_bit_ceil(unsigned n) {
	unsigned c = 1;
	while (c < n)
		c <<= 1;
	int z = 0;
	while (!(c & 1u)) {
		c >>= 1;
		++z;
	}
	return z;
}

struct Trait {
	unsigned variants, transforms;
	int variant_bits, transform_bits;
};

hc_block_props make(uint16_t t0, uint16_t t1, uint16_t t2, uint16_t t3, uint16_t t4, uint16_t t5, uint8_t transparency,
                    uint8_t light, uint8_t collision) {
	hc_block_props p;
	memset(&p, 0, sizeof(p));
	p.tex[0] = t0, p.tex[1] = t1, p.tex[2] = t2, p.tex[3] = t3, p.tex[4] = t4, p.tex[5] = t5;
	p.transparency = transparency;
	p.light_level = light;
	p.collision = collision;
	return p;
}
hc_block_props same(uint16_t t, uint8_t transparency, uint8_t light, uint8_t collision) {
	return make(t, t, t, t, t, t, transparency, light, collision);
}
// BLOCK_TEXTURE_BOT_SIDE_TOP(b, s, t) = {s, s, t, b, s, s}
hc_block_props bot_side_top(uint16_t b, uint16_t s, uint16_t t, uint8_t transparency, uint8_t light, uint8_t collision) {
	return make(s, s, t, b, s, s, transparency, light, collision);
}
hc_block_props none(uint8_t transparency, uint8_t collision) {
	return make(0, 0, 0, 0, 0, 0, transparency, 0, collision);
}

struct StaticMeshes {
	hc_mesh_face *faces;
	uint32_t count;
	// first face of each named mesh
	uint8_t grass_cross[4], dead_bush, apple, red_mushroom, brown_mushroom, cactus, vine[6];
	uint8_t grass_cross_n[4], dead_bush_n, apple_n, red_mushroom_n, brown_mushroom_n, cactus_n, vine_n[6];
};

hc_mesh_face face(uint8_t axis, uint8_t light_face, uint8_t render_face, uint16_t texture, const int v[4][3]) {
	hc_mesh_face f;
	memset(&f, 0, sizeof(f));
	f.axis = axis, f.light_face = light_face, f.render_face = render_face, f.texture = texture;
	for (int i = 0; i < 4; ++i) {
		for (int k = 0; k < 3; ++k)
			f.v[i].pos[k] = (uint8_t)v[i][k];
		f.v[i].ao = 4;
	}
	return f;
}

uint8_t add_cross(StaticMeshes &s, uint16_t tex_id_, int r, int lo, int hi, uint8_t light_face, uint8_t *count) {
	uint8_t first = (uint8_t)s.count;
	const int a = 8 - r, b = 8 + r;
	const int f0[4][3] = {{a, lo, a}, {b, lo, b}, {b, hi, b}, {a, hi, a}};
	const int f1[4][3] = {{a, lo, b}, {b, lo, a}, {b, hi, a}, {a, hi, b}};
	const int f2[4][3] = {{a, hi, a}, {b, hi, b}, {b, lo, b}, {a, lo, a}};
	const int f3[4][3] = {{a, hi, b}, {b, hi, a}, {b, lo, a}, {a, lo, b}};
	s.faces[s.count++] = face(0, light_face, HC_FACE_LEFT, tex(tex_id_), f0);
	s.faces[s.count++] = face(2, light_face, HC_FACE_BACK, tex(tex_id_, HC_TRANS_NEG_U), f1);
	s.faces[s.count++] = face(0, light_face, HC_FACE_RIGHT, tex(tex_id_), f2);
	s.faces[s.count++] = face(2, light_face, HC_FACE_FRONT, tex(tex_id_, HC_TRANS_NEG_U), f3);
	*count = hc_tex_use_transparent_pass(tex_id_) ? 2 : 4;
	return first;
}

uint8_t add_inner_surface(StaticMeshes &s, uint16_t tex_id_, uint8_t fc, uint8_t dist, uint8_t *count) {
	uint8_t first = (uint8_t)s.count;
	int axis = fc >> 1, u = (axis + 1) % 3, v = (axis + 2) % 3;
	int du[3] = {0, 0, 0}, dv[3] = {0, 0, 0}, x[3] = {0, 0, 0};
	if (fc & 1u) {
		du[v] = dv[u] = 16;
		x[axis] = 16 - (int)dist;
	} else {
		dv[v] = du[u] = 16;
		x[axis] = dist;
	}
	int a[4][3], b[4][3];
	for (int k = 0; k < 3; ++k) {
		a[0][k] = x[k], a[1][k] = x[k] + du[k], a[2][k] = x[k] + du[k] + dv[k], a[3][k] = x[k] + dv[k];
		b[0][k] = x[k], b[1][k] = x[k] + dv[k], b[2][k] = x[k] + du[k] + dv[k], b[3][k] = x[k] + du[k];
	}
	s.faces[s.count++] = face((uint8_t)axis, fc, fc, tex(tex_id_), a);
	s.faces[s.count++] = face((uint8_t)axis, fc, (uint8_t)(fc ^ 1u), tex(tex_id_), b);
	*count = hc_tex_use_transparent_pass(tex_id_) ? 1 : 2;
	return first;
}

uint8_t add_cactus(StaticMeshes &s, uint8_t *count) {
	uint8_t first = (uint8_t)s.count;
	const uint16_t t = tex(HC_TEX_CACTUS_SIDE);
	const int r[4][3] = {{15, 0, 16}, {15, 0, 0}, {15, 16, 0}, {15, 16, 16}};
	const int l[4][3] = {{1, 0, 0}, {1, 0, 16}, {1, 16, 16}, {1, 16, 0}};
	const int f[4][3] = {{0, 0, 15}, {16, 0, 15}, {16, 16, 15}, {0, 16, 15}};
	const int k[4][3] = {{16, 0, 1}, {0, 0, 1}, {0, 16, 1}, {16, 16, 1}};
	s.faces[s.count++] = face(0, HC_FACE_RIGHT, HC_FACE_RIGHT, t, r);
	s.faces[s.count++] = face(0, HC_FACE_LEFT, HC_FACE_LEFT, t, l);
	s.faces[s.count++] = face(2, HC_FACE_FRONT, HC_FACE_FRONT, t, f);
	s.faces[s.count++] = face(2, HC_FACE_BACK, HC_FACE_BACK, t, k);
	*count = 4;
	return first;
}

hc_block_props with_mesh(hc_block_props p, uint8_t first, uint8_t count) {
	p.mesh_kind = HC_MESH_STATIC;
	p.mesh_first = first;
	p.mesh_count = count;
	return p;
}

Trait single(unsigned transforms = 0) { return {1, transforms, 0, countr_zero_bit_ceil(transforms)}; }
Trait multi(unsigned variants, unsigned transforms = 0) {
	return {variants, transforms, countr_zero_bit_ceil(variants), countr_zero_bit_ceil(transforms)};
}

Trait trait_of(unsigned id) {
	switch (id) {
	case HC_BLK_GRASS_BLOCK:
	case HC_BLK_GRASS:
		return multi(4);
	case HC_BLK_LEAVES:
	case HC_BLK_PLANK:
		return multi(5);
	case HC_BLK_LOG:
		return multi(5, 3);
	case HC_BLK_VINE:
		return single(6);
	case HC_BLK_FLOWING_WATER:
		return multi(9);
	default:
		return id < HC_BLK_ID_COUNT ? single() : Trait{0, 0, 0, 0};
	}
}

hc_block_props props_of(unsigned id, unsigned variant, unsigned transform, const StaticMeshes &s) {
	static const uint16_t kGrassSide[4] = {HC_TEX_GRASS_PLAIN_SIDE, HC_TEX_GRASS_SAVANNA_SIDE,
	                                       HC_TEX_GRASS_TROPICAL_SIDE, HC_TEX_GRASS_BOREAL_SIDE};
	static const uint16_t kGrassTop[4] = {HC_TEX_GRASS_PLAIN_TOP, HC_TEX_GRASS_SAVANNA_TOP, HC_TEX_GRASS_TROPICAL_TOP,
	                                      HC_TEX_GRASS_BOREAL_TOP};
	// Variant order of leaves/logs/planks: oak, acacia, jungle, spruce, birch.
	static const uint16_t kLeaves[5] = {HC_TEX_OAK_LEAVES, HC_TEX_ACACIA_LEAVES, HC_TEX_JUNGLE_LEAVES,
	                                    HC_TEX_SPRUCE_LEAVES, HC_TEX_BIRCH_LEAVES};
	static const uint16_t kLog[5] = {HC_TEX_OAK_LOG, HC_TEX_ACACIA_LOG, HC_TEX_JUNGLE_LOG, HC_TEX_SPRUCE_LOG,
	                                 HC_TEX_BIRCH_LOG};
	static const uint16_t kLogTop[5] = {HC_TEX_OAK_LOG_TOP, HC_TEX_ACACIA_LOG_TOP, HC_TEX_JUNGLE_LOG_TOP,
	                                    HC_TEX_SPRUCE_LOG_TOP, HC_TEX_BIRCH_LOG_TOP};
	static const uint16_t kPlank[5] = {HC_TEX_OAK_PLANK, HC_TEX_ACACIA_PLANK, HC_TEX_JUNGLE_PLANK,
	                                   HC_TEX_SPRUCE_PLANK, HC_TEX_BIRCH_PLANK};
	switch (id) {
	case HC_BLK_AIR:
		return none(HC_TRANSPARENT, HC_COLLISION_NONE);
	case HC_BLK_STONE:
		return same(HC_TEX_STONE, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_COBBLESTONE:
		return same(HC_TEX_COBBLESTONE, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_DIRT:
		return same(HC_TEX_DIRT, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_GRASS_BLOCK:
		return bot_side_top(HC_TEX_DIRT, kGrassSide[variant], kGrassTop[variant], HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_GRASS:
		return with_mesh(none(HC_TRANSPARENT, HC_COLLISION_NONE), s.grass_cross[variant], s.grass_cross_n[variant]);
	case HC_BLK_SAND:
		return same(HC_TEX_SAND, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_DEAD_BUSH:
		return with_mesh(none(HC_TRANSPARENT, HC_COLLISION_NONE), s.dead_bush, s.dead_bush_n);
	case HC_BLK_GRAVEL:
		return same(HC_TEX_GRAVEL, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_GLASS:
		return same(HC_TEX_GLASS, HC_TRANSPARENT, 0, HC_COLLISION_SOLID);
	case HC_BLK_SNOW:
		return same(HC_TEX_SNOW, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_BLUE_ICE:
		return same(HC_TEX_BLUE_ICE, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_ICE:
		return same(HC_TEX_ICE, HC_SEMI_TRANSPARENT, 0, HC_COLLISION_SOLID);
	case HC_BLK_SANDSTONE:
		return same(HC_TEX_SANDSTONE, HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_WATER:
		return same(HC_TEX_WATER, HC_SEMI_TRANSPARENT, 0, HC_COLLISION_WATER);
	case HC_BLK_FLOWING_WATER: {
		hc_block_props p = none(HC_SEMI_TRANSPARENT, HC_COLLISION_WATER);
		p.mesh_kind = HC_MESH_FLOW;
		p.flow_variant = (uint8_t)variant;
		return p;
	}
	case HC_BLK_LEAVES:
		return same(kLeaves[variant], HC_SEMI_TRANSPARENT, 0, HC_COLLISION_SOLID);
	case HC_BLK_LOG: {
		hc_block_props p =
		    bot_side_top(kLogTop[variant], kLog[variant], kLogTop[variant], HC_OPAQUE, 0, HC_COLLISION_SOLID);
		const uint16_t *t = p.tex;
		if (transform == 0) { // RotateCW(2)
			return make(t[HC_FACE_TOP], t[HC_FACE_BOTTOM], swap_uv(t[HC_FACE_LEFT]), swap_uv(t[HC_FACE_RIGHT]),
			            rot_cw(t[4]), rot_ccw(t[5]), HC_OPAQUE, 0, HC_COLLISION_SOLID);
		} else if (transform == 2) { // RotateCW(0)
			return make(rot_cw(t[0]), rot_ccw(t[1]), t[HC_FACE_FRONT], t[HC_FACE_BACK], t[HC_FACE_BOTTOM],
			            t[HC_FACE_TOP], HC_OPAQUE, 0, HC_COLLISION_SOLID);
		}
		return p;
	}
	case HC_BLK_PLANK:
		return same(kPlank[variant], HC_OPAQUE, 0, HC_COLLISION_SOLID);
	case HC_BLK_APPLE:
		return with_mesh(none(HC_TRANSPARENT, HC_COLLISION_NONE), s.apple, s.apple_n);
	case HC_BLK_CACTUS:
		return with_mesh(bot_side_top(HC_TEX_CACTUS_BOTTOM, 0, HC_TEX_CACTUS_TOP, HC_SEMI_TRANSPARENT, 0,
		                              HC_COLLISION_SOLID),
		                 s.cactus, s.cactus_n);
	case HC_BLK_VINE:
		return with_mesh(none(HC_TRANSPARENT, HC_COLLISION_NONE), s.vine[transform], s.vine_n[transform]);
	case HC_BLK_RED_MUSHROOM:
		return with_mesh(none(HC_TRANSPARENT, HC_COLLISION_NONE), s.red_mushroom, s.red_mushroom_n);
	case HC_BLK_BROWN_MUSHROOM:
		return with_mesh(none(HC_TRANSPARENT, HC_COLLISION_NONE), s.brown_mushroom, s.brown_mushroom_n);
	case HC_BLK_GLOWSTONE:
		return same(HC_TEX_GLOWSTONE, HC_OPAQUE, 15, HC_COLLISION_SOLID);
	default: // unregistered id: the default BlockTrait ("None")
		return none(HC_TRANSPARENT, HC_COLLISION_NONE);
	}
}

} // namespace

extern "C" {

int hc_tex_is_transparent(uint16_t t) {
	uint16_t id = tex_id(t);
	return id < HC_TEX_COUNT ? (int)((kTransparentTex >> id) & 1u) : 0;
}
int hc_tex_is_liquid(uint16_t t) {
	uint16_t id = tex_id(t);
	return id < HC_TEX_COUNT ? (int)((kLiquidTex >> id) & 1u) : 0;
}
int hc_tex_use_transparent_pass(uint16_t t) {
	uint16_t id = tex_id(t);
	return id < HC_TEX_COUNT ? (int)((kTransPassTex >> id) & 1u) : 0;
}

int hc_registry_build(hc_registry *reg) {
	memset(reg, 0, sizeof(*reg));
	StaticMeshes s;
	memset(&s, 0, sizeof(s));
	s.faces = reg->static_faces;
	static const uint16_t kGrassPlant[4] = {HC_TEX_GRASS_PLAIN, HC_TEX_GRASS_SAVANNA, HC_TEX_GRASS_TROPICAL,
	                                        HC_TEX_GRASS_BOREAL};
	for (int v = 0; v < 4; ++v)
		s.grass_cross[v] = add_cross(s, kGrassPlant[v], 8, 0, 16, HC_FACE_TOP, &s.grass_cross_n[v]);
	s.dead_bush = add_cross(s, HC_TEX_DEAD_BUSH, 8, 0, 16, HC_FACE_TOP, &s.dead_bush_n);
	s.apple = add_cross(s, HC_TEX_APPLE, 5, 1, 15, HC_FACE_BOTTOM, &s.apple_n);
	// The mushrooms pass `true` as the light-face template argument, i.e. face 1 (-x).
	s.red_mushroom = add_cross(s, HC_TEX_RED_MUSHROOM, 5, 0, 12, 1, &s.red_mushroom_n);
	s.brown_mushroom = add_cross(s, HC_TEX_BROWN_MUSHROOM, 6, 0, 9, 1, &s.brown_mushroom_n);
	s.cactus = add_cactus(s, &s.cactus_n);
	for (int t = 0; t < 6; ++t)
		s.vine[t] = add_inner_surface(s, HC_TEX_VINE, (uint8_t)t, 1, &s.vine_n[t]);
	reg->static_face_count = s.count;

	for (unsigned raw = 0; raw < 65536u; ++raw) {
		unsigned id = raw & 0xffu, meta = raw >> 8;
		Trait tr = trait_of(id);
		// min<u8>(bits, count - 1), with count 0 wrapping to 255
		unsigned vmax = (uint8_t)(tr.variants - 1u), tmax = (uint8_t)(tr.transforms - 1u);
		unsigned variant = meta & ((1u << tr.variant_bits) - 1u);
		if (variant > vmax)
			variant = vmax;
		unsigned transform = (meta >> tr.variant_bits) & ((1u << tr.transform_bits) - 1u);
		if (transform > tmax)
			transform = tmax;
		hc_block_props p = props_of(id, variant, transform, s);
		p.id = (uint8_t)id;
		reg->props[raw] = p;
	}
	return 0;
}

void hc_flow_mesh(const uint16_t nei[8], uint8_t variant, hc_mesh_face *faces, uint32_t *face_count,
                  uint16_t textures[6]) {
	hc_flow_mesh_impl(nei, variant, faces, face_count, textures);
}

} // extern "C"
