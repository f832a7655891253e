// Seeded synthetic worlds for the chunk relight + mesh path (host C++, no GPU).
//
// The reference's own terrain uses FastNoise2 (client/src/DefaultTerrain.cpp:10-165); these worlds
// instead follow the benchmark specification: a 2D value-noise heightmap (4 octaves, base period 64,
// lacunarity 2, gain 0.5, height 16 + round(12 n)), stone / dirt / grass fill, 5% leaves on
// surface-adjacent air, optional 3D value-noise caves with glowstone, and the per-column sunlight
// height rule of client/src/ChunkFloodSunlightTask.cpp:41-57 cascaded from the top chunk layer.
// All arithmetic is integer (16.16 fixed point) so x86 and aarch64 hosts generate identical bytes.
#include "hc_worldgen.h"

#include "hc_registry.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr int kS = 32;
constexpr int64_t kOne = 1 << 16;

inline uint64_t splitmix64(uint64_t x) {
	x += 0x9e3779b97f4a7c15ull;
	x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
	x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
	return x ^ (x >> 31);
}
inline uint64_t hash4(int64_t a, int64_t b, int64_t c, uint64_t d) {
	uint64_t h = splitmix64((uint64_t)a ^ 0x1234567ull);
	h = splitmix64(h ^ (uint64_t)b);
	h = splitmix64(h ^ (uint64_t)c);
	return splitmix64(h ^ d);
}
// lattice value in [-1, 1] as 16.16
inline int64_t lattice(int64_t a, int64_t b, int64_t c, uint64_t key) {
	return (int64_t)(hash4(a, b, c, key) >> 47) - kOne; // 17 bits -> [0, 2^17) - 2^16
}
// smoothstep of a 16.16 fraction
inline int64_t smooth(int64_t t) { return (t * t / kOne) * (3 * kOne - 2 * t) / kOne; }
inline int64_t lerp(int64_t a, int64_t b, int64_t t) { return a + (b - a) * t / kOne; }
inline int64_t floor_div(int64_t a, int64_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// 2D value noise, fractal sum normalised to [-1, 1] (16.16).
int64_t noise2(int64_t x, int64_t z, uint64_t seed) {
	int64_t sum = 0, amp = kOne, norm = 0;
	int64_t period = 64;
	for (int o = 0; o < 4; ++o) {
		int64_t ix = floor_div(x, period), iz = floor_div(z, period);
		int64_t fx = (x - ix * period) * kOne / period, fz = (z - iz * period) * kOne / period;
		uint64_t key = seed * 0x9e3779b97f4a7c15ull + (uint64_t)o;
		int64_t v00 = lattice(ix, iz, 0, key), v10 = lattice(ix + 1, iz, 0, key);
		int64_t v01 = lattice(ix, iz + 1, 0, key), v11 = lattice(ix + 1, iz + 1, 0, key);
		int64_t sx = smooth(fx), sz = smooth(fz);
		int64_t v = lerp(lerp(v00, v10, sx), lerp(v01, v11, sx), sz);
		sum += v * amp / kOne;
		norm += amp;
		amp /= 2;
		period /= 2;
	}
	return sum * kOne / norm;
}

// 3D value noise (3 octaves, base period 32), in [-1, 1] (16.16).
int64_t noise3(int64_t x, int64_t y, int64_t z, uint64_t seed) {
	int64_t sum = 0, amp = kOne, norm = 0;
	int64_t period = 32;
	for (int o = 0; o < 3; ++o) {
		int64_t ix = floor_div(x, period), iy = floor_div(y, period), iz = floor_div(z, period);
		int64_t fx = (x - ix * period) * kOne / period, fy = (y - iy * period) * kOne / period,
		        fz = (z - iz * period) * kOne / period;
		uint64_t key = (seed ^ 0xc0ffee1234ull) * 0x9e3779b97f4a7c15ull + (uint64_t)o;
		int64_t sx = smooth(fx), sy = smooth(fy), sz = smooth(fz);
		int64_t c[2][2];
		for (int dy = 0; dy < 2; ++dy)
			for (int dz = 0; dz < 2; ++dz) {
				int64_t a = lattice(ix, iy + dy, iz + dz, key ^ 0x55ull), b = lattice(ix + 1, iy + dy, iz + dz, key ^ 0x55ull);
				c[dy][dz] = lerp(a, b, sx);
			}
		int64_t v = lerp(lerp(c[0][0], c[0][1], sz), lerp(c[1][0], c[1][1], sz), sy);
		sum += v * amp / kOne;
		norm += amp;
		amp /= 2;
		period /= 2;
	}
	return sum * kOne / norm;
}

inline int surface_height(int64_t wx, int64_t wz, uint64_t seed) {
	int64_t n = noise2(wx, wz, seed);
	return 16 + (int)floor_div(12 * n + kOne / 2, kOne);
}

inline uint32_t cell_rand(int64_t x, int64_t y, int64_t z, uint64_t seed, uint64_t salt) {
	return (uint32_t)(hash4(x, y, z, seed ^ salt) >> 32);
}
inline bool chance(int64_t x, int64_t y, int64_t z, uint64_t seed, uint64_t salt, uint32_t permille) {
	return cell_rand(x, y, z, seed, salt) % 1000u < permille;
}

// Cave threshold: the 85th percentile of noise3 over a fixed sample (so ~15% of cells carve).
int64_t cave_threshold(uint64_t seed) {
	std::vector<int64_t> v;
	v.reserve(1 << 16);
	for (int i = 0; i < (1 << 16); ++i) {
		uint64_t h = splitmix64(seed ^ (0xabcdull + (uint64_t)i));
		int64_t x = (int64_t)(h & 0xfff), y = (int64_t)((h >> 12) & 0xff), z = (int64_t)((h >> 20) & 0xfff);
		v.push_back(noise3(x, y - 128, z, seed));
	}
	std::nth_element(v.begin(), v.begin() + (v.size() * 85) / 100, v.end());
	return v[(v.size() * 85) / 100];
}

struct Grid {
	const hcw_grid *g;
	uint16_t *blocks;
	int8_t *heights;
	size_t chunk_index(int ix, int iy, int iz) const { return (size_t)ix + (size_t)g->nx * ((size_t)iz + (size_t)g->nz * iy); }
	uint16_t *chunk(int ix, int iy, int iz) const { return blocks + chunk_index(ix, iy, iz) * (size_t)(kS * kS * kS); }
	int8_t *hchunk(int ix, int iy, int iz) const { return heights + chunk_index(ix, iy, iz) * (size_t)(kS * kS); }
};

// Terrain block at a world position: surface fill, caves and glowstone (no leaves).
inline uint16_t terrain_block(int64_t wx, int64_t wy, int64_t wz, int h, const hcw_params &p, int64_t cave_thr) {
	if (wy > h)
		return HC_BLK_AIR;
	if (p.caves && wy < h) {
		if (noise3(wx, wy, wz, p.seed) > cave_thr)
			return chance(wx, wy, wz, p.seed, 0x7011ull, 20) ? (uint16_t)HC_BLK_GLOWSTONE : (uint16_t)HC_BLK_AIR;
	}
	if (wy == h)
		return HC_BLK_GRASS_BLOCK;
	if (wy >= h - 4)
		return HC_BLK_DIRT;
	return HC_BLK_STONE;
}

void fill_terrain_chunk(uint16_t *dst, int64_t cx, int64_t cy, int64_t cz, const hcw_params &p, int64_t cave_thr) {
	int hmap[34][34];
	for (int z = -1; z <= kS; ++z)
		for (int x = -1; x <= kS; ++x)
			hmap[z + 1][x + 1] = surface_height(cx * kS + x, cz * kS + z, p.seed);
	for (int y = 0; y < kS; ++y)
		for (int z = 0; z < kS; ++z)
			for (int x = 0; x < kS; ++x) {
				int64_t wx = cx * kS + x, wy = cy * kS + y, wz = cz * kS + z;
				int h = hmap[z + 1][x + 1];
				uint16_t b = terrain_block(wx, wy, wz, h, p, cave_thr);
				if (b == HC_BLK_AIR && wy > h && p.leaves_permille) {
					// air cell 6-adjacent to a solid terrain block (before leaves are placed)
					bool adj = wy - 1 <= h; // the cell below is terrain
					for (int d = 0; d < 4 && !adj; ++d) {
						static const int kD[4][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}};
						adj = wy <= hmap[z + 1 + kD[d][1]][x + 1 + kD[d][0]];
					}
					if (adj && chance(wx, wy, wz, p.seed, 0x1eafull, (uint32_t)p.leaves_permille))
						b = HC_BLK_LEAVES;
				}
				dst[x + (y * kS + z) * kS] = b;
			}
}

void fill_kind(uint16_t *dst, int kind, int64_t cx, int64_t cy, int64_t cz, const hcw_params &p, int64_t cave_thr) {
	static const uint16_t kFill[12] = {HC_BLK_STONE, HC_BLK_COBBLESTONE, HC_BLK_DIRT, HC_BLK_GRASS_BLOCK,
	                                   HC_BLK_SAND,  HC_BLK_GRAVEL,      HC_BLK_SANDSTONE, HC_BLK_PLANK,
	                                   HC_BLK_GLASS, HC_BLK_ICE,         HC_BLK_LEAVES,    HC_BLK_WATER};
	switch (kind) {
	case HCW_KIND_AIR:
		std::memset(dst, 0, sizeof(uint16_t) * kS * kS * kS);
		break;
	case HCW_KIND_STONE:
		std::fill(dst, dst + kS * kS * kS, (uint16_t)HC_BLK_STONE);
		break;
	case HCW_KIND_TERRAIN:
		fill_terrain_chunk(dst, cx, cy, cz, p, cave_thr);
		break;
	case HCW_KIND_RANDOM:
		for (int y = 0; y < kS; ++y)
			for (int z = 0; z < kS; ++z)
				for (int x = 0; x < kS; ++x) {
					uint32_t r = cell_rand(cx * kS + x, cy * kS + y, cz * kS + z, p.seed, 0x4a4dull);
					dst[x + (y * kS + z) * kS] = (r & 1u) ? kFill[(r >> 1) % 12u] : (uint16_t)HC_BLK_AIR;
				}
		break;
	case HCW_KIND_CHECKER:
		for (int y = 0; y < kS; ++y)
			for (int z = 0; z < kS; ++z)
				for (int x = 0; x < kS; ++x) {
					int64_t s = cx * kS + x + cy * kS + y + cz * kS + z;
					dst[x + (y * kS + z) * kS] = (s & 1) ? (uint16_t)HC_BLK_AIR : (uint16_t)HC_BLK_STONE;
				}
		break;
	}
}

template <typename F> void parallel_for(size_t n, int threads, F f) {
	if (threads <= 1 || n < 2) {
		for (size_t i = 0; i < n; ++i)
			f(i);
		return;
	}
	std::atomic<size_t> next{0};
	std::vector<std::thread> ts;
	for (int t = 0; t < threads; ++t)
		ts.emplace_back([&] {
			for (size_t i; (i = next.fetch_add(1)) < n;)
				f(i);
		});
	for (auto &t : ts)
		t.join();
}

const hc_registry &registry() {
	static hc_registry *r = [] {
		hc_registry *p = new hc_registry;
		hc_registry_build(p);
		return p;
	}();
	return *r;
}

} // namespace

extern "C" {

int hcw_assign_kinds(const hcw_grid *g, const hcw_params *p, uint8_t *kinds) {
	const size_t n = (size_t)g->nx * g->ny * g->nz;
	const int ring = p->air_ring ? 1 : 0;
	std::vector<size_t> inner;
	for (int iy = 0; iy < g->ny; ++iy)
		for (int iz = 0; iz < g->nz; ++iz)
			for (int ix = 0; ix < g->nx; ++ix) {
				size_t i = (size_t)ix + (size_t)g->nx * ((size_t)iz + (size_t)g->nz * iy);
				bool edge = ring && (ix == 0 || iy == 0 || iz == 0 || ix == g->nx - 1 || iy == g->ny - 1 || iz == g->nz - 1);
				kinds[i] = edge ? HCW_KIND_AIR : (uint8_t)p->default_kind;
				if (!edge)
					inner.push_back(i);
			}
	if (!p->mixture)
		return 0;
	// seeded mixture: 30% air, 20% stone, 35% terrain, 10% random fill, 5% checkerboard
	const uint32_t pct[5] = {30, 20, 35, 10, 5};
	const uint8_t kind[5] = {HCW_KIND_AIR, HCW_KIND_STONE, HCW_KIND_TERRAIN, HCW_KIND_RANDOM, HCW_KIND_CHECKER};
	std::vector<uint8_t> list;
	list.reserve(inner.size());
	size_t acc = 0;
	uint32_t cum = 0;
	for (int k = 0; k < 5; ++k) {
		cum += pct[k];
		size_t upto = (inner.size() * cum) / 100;
		for (; acc < upto; ++acc)
			list.push_back(kind[k]);
	}
	for (uint64_t i = list.size(); i > 1; --i) { // Fisher-Yates
		uint64_t j = splitmix64(p->seed ^ (0x5eedull + i)) % i;
		std::swap(list[i - 1], list[j]);
	}
	for (size_t i = 0; i < inner.size(); ++i)
		kinds[inner[i]] = list[i];
	(void)n;
	return 0;
}

int hcw_generate(const hcw_grid *g, const hcw_params *p, const uint8_t *kinds, uint16_t *blocks, int8_t *heights,
                 int threads) {
	if (!g || !p || !kinds || !blocks || !heights || g->nx <= 0 || g->ny <= 0 || g->nz <= 0)
		return -1;
	Grid grid{g, blocks, heights};
	const int64_t thr = p->caves ? cave_threshold(p->seed) : 0;
	const size_t n = (size_t)g->nx * g->ny * g->nz;
	parallel_for(n, threads, [&](size_t i) {
		int ix = (int)(i % g->nx), iz = (int)((i / g->nx) % g->nz), iy = (int)(i / ((size_t)g->nx * g->nz));
		fill_kind(grid.chunk(ix, iy, iz), kinds[i], g->cx0 + ix, g->cy0 + iy, g->cz0 + iz, *p, thr);
	});
	hcw_recompute_heights(g, kinds, p->air_ring, blocks, heights, threads);
	return 0;
}

// Sunlight heights (ChunkFloodSunlightTask.cpp:41-57), cascading from the top chunk layer down:
// a column is dark (32) if the chunk above has a positive height there; otherwise its height is
// one above the highest block that does not pass vertical light. Air-ring chunks stay lit (0).
int hcw_recompute_heights(const hcw_grid *g, const uint8_t *kinds, int air_ring, const uint16_t *blocks, int8_t *heights,
                          int threads) {
	const hc_registry &r = registry();
	Grid grid{g, const_cast<uint16_t *>(blocks), heights};
	const size_t cols = (size_t)g->nx * g->nz;
	parallel_for(cols, threads, [&](size_t c) {
		int ix = (int)(c % g->nx), iz = (int)(c / g->nx);
		for (int iy = g->ny - 1; iy >= 0; --iy) {
			const uint16_t *b = grid.chunk(ix, iy, iz);
			int8_t *h = grid.hchunk(ix, iy, iz);
			size_t ci = grid.chunk_index(ix, iy, iz);
			bool ring = air_ring && kinds && kinds[ci] == HCW_KIND_AIR &&
			            (ix == 0 || iy == 0 || iz == 0 || ix == g->nx - 1 || iy == g->ny - 1 || iz == g->nz - 1);
			const int8_t *up = iy + 1 < g->ny ? grid.hchunk(ix, iy + 1, iz) : nullptr;
			for (int xz = 0; xz < kS * kS; ++xz) {
				if (ring) {
					h[xz] = 0;
					continue;
				}
				if (up && up[xz] > 0) {
					h[xz] = kS;
					continue;
				}
				int y = kS - 1;
				while (y >= 0 && r.props[b[xz + y * kS * kS]].transparency == HC_TRANSPARENT)
					--y;
				h[xz] = (int8_t)(y + 1);
			}
		}
	});
	return 0;
}

// 27-neighbour chunk indices of a chunk in neighbour-index order (centre = 26,
// common/include/common/Position.hpp:146-152), or -1 where the neighbour lies outside the grid.
int hcw_neighbours(const hcw_grid *g, int ix, int iy, int iz, int32_t *out27) {
	static const int kRev[3] = {1, -1, 0};
	for (int i = 0; i < 27; ++i) {
		int dz = kRev[i % 3], dy = kRev[(i / 3) % 3], dx = kRev[i / 9];
		int x = ix + dx, y = iy + dy, z = iz + dz;
		if (x < 0 || y < 0 || z < 0 || x >= g->nx || y >= g->ny || z >= g->nz)
			out27[i] = -1;
		else
			out27[i] = (int32_t)((size_t)x + (size_t)g->nx * ((size_t)z + (size_t)g->nz * y));
	}
	return 0;
}

} // extern "C"
