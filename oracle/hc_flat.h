// Flat, reference-ordered mesh output used by the CPU oracle and by the reference harness.
//
// TEST INFRASTRUCTURE. Nothing in the product links this header.
//
// The reference returns std::vector<BlockMesh> (client/include/client/BlockVertex.hpp:20-25;
// order from client/include/client/BlockMeshAlgo.hpp:494-521). Here the meshes are concatenated in
// that order: mesh i owns the next meshes[i*9+0] vertices and meshes[i*9+1] indices.
#pragma once
#include <stdint.h>

#define HC_FLAT_MESH_WORDS 9 // vertex_count, index_count, aabb_min[3], aabb_max[3], transparent

typedef struct hc_flat_meshes {
	uint32_t mesh_cap, vertex_cap, index_cap;       // capacities (in meshes, vertices, indices)
	uint32_t mesh_count, vertex_count, index_count; // written sizes (required sizes on overflow)
	uint32_t *meshes;                               // mesh_cap * HC_FLAT_MESH_WORDS
	uint32_t *vertices;                             // vertex_cap * 2 (the two packed words)
	uint16_t *indices;                              // index_cap
} hc_flat_meshes;
