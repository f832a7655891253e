// Block and texture registry of HyperCraft, restated as plain data for the GB300 mesher.
//
// A block is a uint16 `raw = id | meta << 8` (block/include/block/Block.hpp:22-33; the
// little-endian {m_id, m_meta} layout applies because common/Endian.hpp is never included).
// Its property row is what the reference's generated 65,536-entry table holds
// (block/generator/Block.cpp.in:9-27, driven by the per-id traits in block/block/*.hpp):
// six face textures, transparency, light level, collision and an optional custom mesh.
//
// This header restates that table from the trait definitions; the row for every raw value is
// pinned against a dump of the reference's own compiled table (tests/golden/registry_*).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Texture ids (texture/register/block_textures, enum order). 13-bit id, 3-bit transform.
enum {
	HC_TEX_NONE = 0,
	HC_TEX_STONE = 1,
	HC_TEX_COBBLESTONE = 2,
	HC_TEX_DIRT = 3,
	HC_TEX_GRASS_PLAIN = 4,
	HC_TEX_GRASS_PLAIN_TOP = 5,
	HC_TEX_GRASS_PLAIN_SIDE = 6,
	HC_TEX_GRASS_SAVANNA = 7,
	HC_TEX_GRASS_SAVANNA_TOP = 8,
	HC_TEX_GRASS_SAVANNA_SIDE = 9,
	HC_TEX_GRASS_TROPICAL = 10,
	HC_TEX_GRASS_TROPICAL_TOP = 11,
	HC_TEX_GRASS_TROPICAL_SIDE = 12,
	HC_TEX_GRASS_BOREAL = 13,
	HC_TEX_GRASS_BOREAL_TOP = 14,
	HC_TEX_GRASS_BOREAL_SIDE = 15,
	HC_TEX_SAND = 16,
	HC_TEX_GRAVEL = 17,
	HC_TEX_GLASS = 18,
	HC_TEX_SNOW = 19,
	HC_TEX_BLUE_ICE = 20,
	HC_TEX_ICE = 21,
	HC_TEX_SANDSTONE = 22,
	HC_TEX_WATER = 23,
	HC_TEX_ACACIA_LEAVES = 24,
	HC_TEX_ACACIA_LOG = 25,
	HC_TEX_ACACIA_LOG_TOP = 26,
	HC_TEX_ACACIA_PLANK = 27,
	HC_TEX_JUNGLE_LEAVES = 28,
	HC_TEX_JUNGLE_LOG = 29,
	HC_TEX_JUNGLE_LOG_TOP = 30,
	HC_TEX_JUNGLE_PLANK = 31,
	HC_TEX_OAK_LEAVES = 32,
	HC_TEX_OAK_LOG = 33,
	HC_TEX_OAK_LOG_TOP = 34,
	HC_TEX_OAK_PLANK = 35,
	HC_TEX_SPRUCE_LEAVES = 36,
	HC_TEX_SPRUCE_LOG = 37,
	HC_TEX_SPRUCE_LOG_TOP = 38,
	HC_TEX_SPRUCE_PLANK = 39,
	HC_TEX_BIRCH_LEAVES = 40,
	HC_TEX_BIRCH_LOG = 41,
	HC_TEX_BIRCH_LOG_TOP = 42,
	HC_TEX_BIRCH_PLANK = 43,
	HC_TEX_DEAD_BUSH = 44,
	HC_TEX_VINE = 45,
	HC_TEX_APPLE = 46,
	HC_TEX_CACTUS_TOP = 47,
	HC_TEX_CACTUS_SIDE = 48,
	HC_TEX_CACTUS_BOTTOM = 49,
	HC_TEX_RED_MUSHROOM = 50,
	HC_TEX_BROWN_MUSHROOM = 51,
	HC_TEX_GLOWSTONE = 52,
	HC_TEX_COUNT = 53
};

// Texture transform bits (texture/include/texture/BlockTexture.hpp:15).
enum { HC_TRANS_SWAP_UV = 1, HC_TRANS_NEG_U = 2, HC_TRANS_NEG_V = 4 };

// Block ids (block/register/blocks, enum order).
enum {
	HC_BLK_AIR = 0,
	HC_BLK_STONE = 1,
	HC_BLK_COBBLESTONE = 2,
	HC_BLK_DIRT = 3,
	HC_BLK_GRASS_BLOCK = 4,
	HC_BLK_GRASS = 5,
	HC_BLK_SAND = 6,
	HC_BLK_DEAD_BUSH = 7,
	HC_BLK_GRAVEL = 8,
	HC_BLK_GLASS = 9,
	HC_BLK_SNOW = 10,
	HC_BLK_BLUE_ICE = 11,
	HC_BLK_ICE = 12,
	HC_BLK_SANDSTONE = 13,
	HC_BLK_WATER = 14,
	HC_BLK_FLOWING_WATER = 15,
	HC_BLK_LEAVES = 16,
	HC_BLK_LOG = 17,
	HC_BLK_PLANK = 18,
	HC_BLK_APPLE = 19,
	HC_BLK_CACTUS = 20,
	HC_BLK_VINE = 21,
	HC_BLK_RED_MUSHROOM = 22,
	HC_BLK_BROWN_MUSHROOM = 23,
	HC_BLK_GLOWSTONE = 24,
	HC_BLK_ID_COUNT = 25
};

// Transparency and collision enums (block/include/block/BlockProperty.hpp:15-16).
enum { HC_OPAQUE = 0, HC_SEMI_TRANSPARENT = 1, HC_TRANSPARENT = 2 };
enum { HC_COLLISION_NONE = 0, HC_COLLISION_SOLID = 1, HC_COLLISION_WATER = 2 };

// Custom-mesh kinds. A static mesh is a fixed face list; a flow mesh is computed from the
// eight horizontal neighbours (block/block/public/Liquid.hpp:156-302).
enum { HC_MESH_NONE = 0, HC_MESH_STATIC = 1, HC_MESH_FLOW = 2 };

// Block faces (block/include/block/BlockFace.hpp:9-11): +x, -x, +y, -y, +z, -z.
enum { HC_FACE_RIGHT = 0, HC_FACE_LEFT = 1, HC_FACE_TOP = 2, HC_FACE_BOTTOM = 3, HC_FACE_FRONT = 4, HC_FACE_BACK = 5 };

// One custom-mesh vertex: position in 1/16 voxel units and an AO code (4 = interpolated).
typedef struct hc_mesh_vertex {
	uint8_t pos[3];
	uint8_t ao;
} hc_mesh_vertex;

// One custom-mesh face (block/include/block/BlockMesh.hpp:28-33).
typedef struct hc_mesh_face {
	uint8_t axis, light_face, render_face, pad;
	uint16_t texture, pad2;
	hc_mesh_vertex v[4];
} hc_mesh_face;

#define HC_MAX_MESH_FACES 16
#define HC_MAX_STATIC_FACES 256

// Property row of one raw block value.
typedef struct hc_block_props {
	uint16_t tex[6];
	uint8_t transparency, light_level, collision, mesh_kind;
	uint8_t mesh_first, mesh_count; // static face range in hc_registry.static_faces
	uint8_t flow_variant;           // clamped variant of a flowing liquid (0..8)
	uint8_t id;                     // block id (low byte of raw)
} hc_block_props;

typedef struct hc_registry {
	hc_block_props props[65536];
	hc_mesh_face static_faces[HC_MAX_STATIC_FACES];
	uint32_t static_face_count;
} hc_registry;

// Fills *reg. Deterministic; returns 0.
int hc_registry_build(hc_registry *reg);

// Texture flag queries (texture/internal/generated/block_texture_transparency.inl).
int hc_tex_is_transparent(uint16_t tex);
int hc_tex_is_liquid(uint16_t tex);
int hc_tex_use_transparent_pass(uint16_t tex);

// Flowing-liquid dynamic mesh (block/block/public/Liquid.hpp:156-282): given the raw values of
// the eight horizontal neighbours in fetch order and the clamped variant, writes the faces and
// the six per-face textures that replace the block's own.
void hc_flow_mesh(const uint16_t nei[8], uint8_t variant, hc_mesh_face *faces, uint32_t *face_count,
                  uint16_t textures[6]);

#ifdef __cplusplus
}
#endif
