// Seeded synthetic chunk grids (host only). Chunk (ix, iy, iz) of a grid is stored at index
// ix + nx * (iz + nz * iy); each chunk is 32^3 uint16 blocks (x + (y*32 + z)*32) followed in a
// separate array by 32^2 int8 sunlight heights (x + z*32), the reference's own chunk layout
// (client/include/client/Chunk.hpp:95-96).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { HCW_KIND_AIR = 0, HCW_KIND_STONE = 1, HCW_KIND_TERRAIN = 2, HCW_KIND_RANDOM = 3, HCW_KIND_CHECKER = 4 };

typedef struct hcw_grid {
	int32_t nx, ny, nz;    // chunks per axis
	int32_t cx0, cy0, cz0; // chunk coordinate of grid cell (0, 0, 0)
} hcw_grid;

typedef struct hcw_params {
	uint64_t seed;
	int32_t caves;           // carve 3D value-noise caves (~15% of underground) with 2% glowstone
	int32_t leaves_permille; // leaves on surface-adjacent air (50 = 5%)
	int32_t air_ring;        // outermost chunk layer is all air and fully lit
	int32_t mixture;         // assign kinds by the seeded 30/20/35/10/5 mixture
	int32_t default_kind;    // kind of non-ring chunks when mixture == 0
} hcw_params;

int hcw_assign_kinds(const hcw_grid *g, const hcw_params *p, uint8_t *kinds);
int hcw_generate(const hcw_grid *g, const hcw_params *p, const uint8_t *kinds, uint16_t *blocks, int8_t *heights,
                 int threads);
int hcw_recompute_heights(const hcw_grid *g, const uint8_t *kinds, int air_ring, const uint16_t *blocks,
                          int8_t *heights, int threads);
int hcw_neighbours(const hcw_grid *g, int ix, int iy, int iz, int32_t *out27);

#ifdef __cplusplus
}
#endif
