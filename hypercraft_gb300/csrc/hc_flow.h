// Flowing-liquid dynamic mesh, shared by the host registry and the device mesher.
//
// Restates block/block/public/Liquid.hpp:151-282 (get_flow_height, flow_mesh_gen<WaterTrait, Variant>) for water
// (Water.hpp:5-14): neighbour heights from the eight horizontal neighbours in fetch order
// (-1,-1) (0,-1) (1,-1) (-1,0) (1,0) (-1,1) (0,1) (1,1) as (dx, dz), corner heights, the sloped top
// face, up to four side faces, and the six textures that replace the block's own face textures.
// Integer types follow the reference: heights are int8, a flowing neighbour's height is
// uint8(max(meta * 2, 1)) reinterpreted as int8, corner heights are uint8.
#pragma once
#include <stdint.h>

#include "hc_registry.h"

#if defined(__CUDACC__)
#define HC_HD __host__ __device__ __forceinline__
#else
#define HC_HD inline
#endif

HC_HD int8_t hc_flow_nei_height(uint16_t raw) {
	unsigned id = raw & 0xffu;
	if (id == HC_BLK_WATER)
		return 16;
	if (id == HC_BLK_FLOWING_WATER) {
		unsigned h = (raw >> 8) * 2u;
		return (int8_t)(uint8_t)(h > 1u ? h : 1u);
	}
	return id != HC_BLK_AIR ? (int8_t)-1 : (int8_t)0;
}

HC_HD uint8_t hc_flow_corner(int8_t nb, int8_t a, int8_t b, int8_t c) {
	int8_t m1 = nb > a ? nb : a;
	int8_t m2 = b > c ? b : c;
	uint8_t mx = (uint8_t)(m1 > m2 ? m1 : m2);
	if (mx != 16 && (nb == 0) + (a == 0) + (b == 0) + (c == 0) >= 3)
		return 0;
	return mx;
}

HC_HD bool hc_flow_is_liquid(uint16_t raw) {
	unsigned id = raw & 0xffu;
	return id == HC_BLK_WATER || id == HC_BLK_FLOWING_WATER;
}

HC_HD void hc_flow_face(hc_mesh_face *f, uint8_t axis, uint8_t face, const uint8_t v[4][3]) {
	f->axis = axis, f->light_face = face, f->render_face = face, f->pad = 0;
	f->texture = HC_TEX_WATER, f->pad2 = 0;
	for (int i = 0; i < 4; ++i) {
		f->v[i].pos[0] = v[i][0], f->v[i].pos[1] = v[i][1], f->v[i].pos[2] = v[i][2];
		f->v[i].ao = 4;
	}
}

// faces may be null when only the count and the textures are wanted.
HC_HD void hc_flow_mesh_impl(const uint16_t nei[8], uint8_t variant, hc_mesh_face *faces, uint32_t *face_count,
                             uint16_t textures[6]) {
	const uint16_t kFlowTex = HC_TEX_WATER, kNone = HC_TEX_NONE;
	int8_t nh[8];
	for (int i = 0; i < 8; ++i)
		nh[i] = hc_flow_nei_height(nei[i]);
	const int8_t nb = (int8_t)(uint8_t)(variant * 2u > 1u ? variant * 2u : 1u);
	const uint8_t h0 = hc_flow_corner(nb, nh[0], nh[1], nh[3]), h1 = hc_flow_corner(nb, nh[1], nh[2], nh[4]);
	const uint8_t h2 = hc_flow_corner(nb, nh[3], nh[5], nh[6]), h3 = hc_flow_corner(nb, nh[4], nh[6], nh[7]);
	if (h0 == 16 && h1 == 16 && h2 == 16 && h3 == 16) {
		*face_count = 0;
		for (int i = 0; i < 6; ++i)
			textures[i] = kFlowTex;
		return;
	}
	uint32_t n = 0;
	if (faces) {
		const uint8_t v[4][3] = {{0, h0, 0}, {0, h2, 16}, {16, h3, 16}, {16, h1, 0}};
		hc_flow_face(faces + n, 1, HC_FACE_TOP, v);
	}
	++n;
	const bool left_full = h0 == 16 && h2 == 16, left_empty = h0 == 0 && h2 == 0;
	const bool right_full = h1 == 16 && h3 == 16, right_empty = h1 == 0 && h3 == 0;
	const bool front_full = h2 == 16 && h3 == 16, front_empty = h2 == 0 && h3 == 0;
	const bool back_full = h0 == 16 && h1 == 16, back_empty = h0 == 0 && h1 == 0;
	if (!left_full && !left_empty && !hc_flow_is_liquid(nei[3])) {
		if (faces) {
			const uint8_t v[4][3] = {{0, h0, 0}, {0, 0, 0}, {0, 0, 16}, {0, h2, 16}};
			hc_flow_face(faces + n, 0, HC_FACE_LEFT, v);
		}
		++n;
	}
	if (!right_full && !right_empty && !hc_flow_is_liquid(nei[4])) {
		if (faces) {
			const uint8_t v[4][3] = {{16, 0, 0}, {16, h1, 0}, {16, h3, 16}, {16, 0, 16}};
			hc_flow_face(faces + n, 0, HC_FACE_RIGHT, v);
		}
		++n;
	}
	if (!back_full && !back_empty && !hc_flow_is_liquid(nei[1])) {
		if (faces) {
			const uint8_t v[4][3] = {{0, 0, 0}, {0, h0, 0}, {16, h1, 0}, {16, 0, 0}};
			hc_flow_face(faces + n, 2, HC_FACE_BACK, v);
		}
		++n;
	}
	if (!front_full && !front_empty && !hc_flow_is_liquid(nei[6])) {
		if (faces) {
			const uint8_t v[4][3] = {{0, h2, 16}, {0, 0, 16}, {16, 0, 16}, {16, h3, 16}};
			hc_flow_face(faces + n, 2, HC_FACE_FRONT, v);
		}
		++n;
	}
	*face_count = n;
	textures[HC_FACE_TOP] = kNone;
	textures[HC_FACE_LEFT] = left_full ? kFlowTex : kNone;
	textures[HC_FACE_RIGHT] = right_full ? kFlowTex : kNone;
	textures[HC_FACE_FRONT] = front_full ? kFlowTex : kNone;
	textures[HC_FACE_BACK] = back_full ? kFlowTex : kNone;
	textures[HC_FACE_BOTTOM] = kFlowTex;
}
