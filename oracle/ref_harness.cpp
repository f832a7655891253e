// Harness around the reference's own relight and mesher templates.
//
// TEST INFRASTRUCTURE. It is compiled only where the reference sources are present (see
// oracle/Makefile.ref), into oracle/_ref/, and is used to pin the CPU oracle and the registry
// restatement. It includes the reference's headers unmodified; the code below only restates
// the glue of client/src/ChunkMeshTask.cpp:41-122 over plain arrays, because the reference's
// Chunk class pulls in the Vulkan renderer (client/include/client/Chunk.hpp:10-11).
#include <client/BlockLightAlgo.hpp>
#include <client/BlockMeshAlgo.hpp>
#include <common/Position.hpp>

#include <atomic>
#include <cstring>
#include <thread>
#include <map>
#include <vector>

#include "hc_flat.h"

using namespace hc;
using namespace hc::client;

namespace {

// ChunkMeshTask.inl:53-56: the light algorithm of the kMesh runner.
using LightAlgo = BlockLightAlgo<BlockAlgoConfig<InnerPos1, BlockAlgoBound<InnerPos1>{-1, -1, -1, (InnerPos1)kChunkSize + 1,
                                                                                     (InnerPos1)kChunkSize + 1,
                                                                                     (InnerPos1)kChunkSize + 1}>,
                                 14>;
// ChunkMeshTask.cpp:113-115: the mesher configuration.
using MeshAlgo = BlockMeshAlgo<
    BlockAlgoConfig<InnerPos1, BlockAlgoBound<InnerPos1>{0, 0, 0, kChunkSize, kChunkSize, kChunkSize}, kBlockAlgoSwizzleYZX>>;

constexpr uint32_t kExt = kChunkSize + 30;

// ChunkMeshTask.cpp:10-12.
template <std::signed_integral T> inline uint32_t ext_index(T x, T y, T z) {
	return x + 15 + ((z + 15) + (y + 15) * kExt) * kExt;
}

struct Neighbours {
	const uint16_t *const *blocks;
	const int8_t *const *heights;
	// Chunk::GetBlockFromNeighbour (Chunk.hpp:57-59) on chunk GetBlockNeighbourIndex(x, y, z).
	template <typename T> block::Block get_block(T x, T y, T z) const {
		uint32_t n = GetBlockChunkNeighbourIndex(x, y, z);
		block::Block b;
		b.SetData(blocks[n][InnerIndex3FromPos((x + kChunkSize) % kChunkSize, (y + kChunkSize) % kChunkSize,
		                                       (z + kChunkSize) % kChunkSize)]);
		return b;
	}
	// Chunk::GetSunlightFromNeighbour (Chunk.hpp:77-79 -> 74-76).
	template <typename T> bool get_sunlight(T x, T y, T z) const {
		uint32_t n = GetBlockChunkNeighbourIndex(x, y, z);
		uint32_t ux = (x + kChunkSize) % kChunkSize, uy = (y + kChunkSize) % kChunkSize,
		         uz = (z + kChunkSize) % kChunkSize;
		return uy >= heights[n][InnerIndex2FromPos(ux, uz)];
	}
};

struct Runner {
	LightAlgo::Queue sun_entries, torch_entries;
	block::Light light[kExt * kExt * kExt]{};

	// ChunkMeshTask.cpp:48-111.
	void relight(const Neighbours &nb) {
		for (InnerPos1 y = -15; y < (InnerPos1)kChunkSize + 15; ++y)
			for (InnerPos1 z = -15; z < (InnerPos1)kChunkSize + 15; ++z)
				for (InnerPos1 x = -15; x < (InnerPos1)kChunkSize + 15; ++x) {
					block::Light l = {};
					l.SetTorchlight(nb.get_block(x, y, z).GetLightLevel());
					l.SetSunlight(nb.get_sunlight(x, y, z) ? 15 : 0);
					light[ext_index(x, y, z)] = l;
					if (LightAlgo::IsBorderLightInterfere(x, y, z, l.GetTorchlight()))
						torch_entries.push({{x, y, z}, l.GetTorchlight()});
				}
		for (InnerPos1 y = -15; y < (InnerPos1)kChunkSize + 15; ++y)
			for (InnerPos1 z = -15; z < (InnerPos1)kChunkSize + 15; ++z)
				for (InnerPos1 x = -15; x < (InnerPos1)kChunkSize + 15; ++x) {
					auto s = light[ext_index(x, y, z)].GetSunlight();
					if (LightAlgo::IsBorderLightInterfere(x, y, z, s)) {
						const auto lit = [&](InnerPos1 a, InnerPos1 b, InnerPos1 c) {
							return light[ext_index(a, b, c)].GetSunlight() == 15;
						};
						if ((x == -15 || lit(InnerPos1(x - 1), y, z)) &&
						    (x == (InnerPos1)kChunkSize + 14 || lit(InnerPos1(x + 1), y, z)) &&
						    (z == -15 || lit(x, y, InnerPos1(z - 1))) &&
						    (z == (InnerPos1)kChunkSize + 14 || lit(x, y, InnerPos1(z + 1))) &&
						    (y == -15 || lit(x, InnerPos1(y - 1), z)) &&
						    (y == (InnerPos1)kChunkSize + 14 || lit(x, InnerPos1(y + 1), z)))
							continue;
						sun_entries.push({{x, y, z}, s});
					}
				}
		LightAlgo algo{};
		const auto get_block = [&nb](auto x, auto y, auto z) -> block::Block { return nb.get_block(x, y, z); };
		algo.PropagateLight(
		    &sun_entries, get_block,
		    [this](auto x, auto y, auto z) -> block::LightLvl { return light[ext_index(x, y, z)].GetSunlight(); },
		    [this](auto x, auto y, auto z, block::LightLvl lvl) { light[ext_index(x, y, z)].SetSunlight(lvl); });
		algo.PropagateLight(
		    &torch_entries, get_block,
		    [this](auto x, auto y, auto z) -> block::LightLvl { return light[ext_index(x, y, z)].GetTorchlight(); },
		    [this](auto x, auto y, auto z, block::LightLvl lvl) { light[ext_index(x, y, z)].SetTorchlight(lvl); });
	}

	// ChunkMeshTask.cpp:113-122.
	std::vector<BlockMesh> mesh(const Neighbours &nb) {
		return MeshAlgo{}.Generate(
		    [&nb](auto x, auto y, auto z) -> block::Block { return nb.get_block(x, y, z); },
		    [this](auto x, auto y, auto z) -> block::Light { return light[ext_index(x, y, z)]; });
	}
};

int write_flat(const std::vector<BlockMesh> &meshes, hc_flat_meshes *out) {
	uint32_t nv = 0, ni = 0;
	for (const auto &m : meshes)
		nv += (uint32_t)m.vertices.size(), ni += (uint32_t)m.indices.size();
	out->mesh_count = (uint32_t)meshes.size();
	out->vertex_count = nv;
	out->index_count = ni;
	if (meshes.size() > out->mesh_cap || nv > out->vertex_cap || ni > out->index_cap)
		return 1;
	uint32_t vo = 0, io = 0;
	for (size_t i = 0; i < meshes.size(); ++i) {
		const auto &m = meshes[i];
		uint32_t *w = out->meshes + i * HC_FLAT_MESH_WORDS;
		w[0] = (uint32_t)m.vertices.size();
		w[1] = (uint32_t)m.indices.size();
		for (int k = 0; k < 3; ++k) {
			w[2 + k] = m.aabb.GetMin()[k];
			w[5 + k] = m.aabb.GetMax()[k];
		}
		w[8] = m.transparent ? 1u : 0u;
		for (const auto &v : m.vertices) {
			out->vertices[2 * vo] = v.x10_y10_z10_axis2;
			out->vertices[2 * vo + 1] = v.tex10_trans3_face3_ao2_sl6_tl6;
			++vo;
		}
		for (auto idx : m.indices)
			out->indices[io++] = idx;
	}
	return 0;
}

thread_local Runner *t_runner = nullptr;
Runner &runner() {
	if (!t_runner)
		t_runner = new Runner();
	return *t_runner;
}

void encode_face(const block::BlockMeshFace &f, uint8_t *dst24) {
	std::memset(dst24, 0, 24);
	dst24[0] = f.axis;
	dst24[1] = f.light_face;
	dst24[2] = f.render_face;
	uint16_t t = f.texture.GetData();
	std::memcpy(dst24 + 4, &t, 2);
	for (int i = 0; i < 4; ++i) {
		dst24[8 + 4 * i + 0] = f.vertices[i].x;
		dst24[8 + 4 * i + 1] = f.vertices[i].y;
		dst24[8 + 4 * i + 2] = f.vertices[i].z;
		dst24[8 + 4 * i + 3] = f.vertices[i].ao;
	}
}

} // namespace

extern "C" {

// Relights one chunk's 62^3 window exactly as the kMesh runner does and copies it out
// (index x+15 + ((z+15) + (y+15)*62)*62, sun in the low nibble, torch in the high nibble).
void hcref_relight_window(const uint16_t *const *blocks, const int8_t *const *heights, uint8_t *light62) {
	Neighbours nb{blocks, heights};
	Runner &r = runner();
	r.relight(nb);
	for (uint32_t i = 0; i < kExt * kExt * kExt; ++i)
		light62[i] = r.light[i].GetData();
}

// Relight + mesh of the centre chunk (neighbour index 26), reference order.
int hcref_mesh_chunk(const uint16_t *const *blocks, const int8_t *const *heights, hc_flat_meshes *out) {
	Neighbours nb{blocks, heights};
	Runner &r = runner();
	r.relight(nb);
	return write_flat(r.mesh(nb), out);
}

// Block table dump: textures (6 x u16), transparency, light level, collision, and a mesh key
// per raw value: 0 = none, 1 + k = k-th distinct static mesh, 0xffff = dynamic (flow) mesh.
// Static meshes are written as face_count then 24-byte faces (same layout as hc_mesh_face).
int hcref_dump_registry(uint16_t *tex6, uint8_t *transparency, uint8_t *light, uint8_t *collision, uint16_t *mesh_key,
                        uint8_t *mesh_faces, uint32_t mesh_faces_cap, uint32_t *mesh_count) {
	std::map<const block::BlockMesh *, uint16_t> keys;
	uint32_t nmesh = 0;
	for (uint32_t raw = 0; raw < 65536u; ++raw) {
		block::Block b;
		b.SetData((uint16_t)raw);
		for (int f = 0; f < 6; ++f)
			tex6[raw * 6 + f] = b.GetTexture((block::BlockFace)f).GetData();
		transparency[raw] = (uint8_t)b.GetTransparency();
		light[raw] = b.GetLightLevel();
		collision[raw] = (uint8_t)b.GetCollision();
		const block::BlockMesh *m = b.GetCustomMesh();
		if (!m) {
			mesh_key[raw] = 0;
		} else if (m->p_dynamic_mesh_func) {
			mesh_key[raw] = 0xffff;
		} else {
			auto it = keys.find(m);
			if (it == keys.end()) {
				if ((nmesh + 1) * (1 + 16 * 24) > mesh_faces_cap)
					return 1;
				uint8_t *dst = mesh_faces + nmesh * (1 + 16 * 24);
				dst[0] = (uint8_t)m->face_count;
				for (uint32_t f = 0; f < m->face_count; ++f)
					encode_face(m->faces[f], dst + 1 + f * 24);
				it = keys.emplace(m, (uint16_t)(++nmesh)).first;
			}
			mesh_key[raw] = it->second;
		}
	}
	*mesh_count = nmesh;
	return 0;
}

// Runs the dynamic mesh function of `self_raw` (a flowing liquid) on eight neighbour values.
int hcref_flow_mesh(uint16_t self_raw, const uint16_t *nei8, uint8_t *faces_out /*16*24*/, uint32_t *face_count,
                    uint16_t *tex_out6) {
	block::Block b;
	b.SetData(self_raw);
	const block::BlockMesh *m = b.GetCustomMesh();
	if (!m || !m->p_dynamic_mesh_func)
		return 1;
	block::Block nei[block::kBlockDynamicMeshMaxNeighbours];
	for (int i = 0; i < 8; ++i)
		nei[i].SetData(nei8[i]);
	block::BlockMeshFace faces[block::kBlockMeshMaxFaceCount];
	uint32_t count = m->face_count;
	std::array<texture::BlockTexture, 6> tex{};
	bool dyn = false;
	m->p_dynamic_mesh_func(nei, faces, &count, tex.data(), &dyn);
	*face_count = count;
	for (uint32_t f = 0; f < count; ++f)
		encode_face(faces[f], faces_out + f * 24);
	for (int f = 0; f < 6; ++f)
		tex_out6[f] = dyn ? tex[f].GetData() : 0xffff;
	return 0;
}

// Neighbour fetch offsets of the dynamic mesh (dx, dy, dz triples).
int hcref_flow_fetch_offsets(uint16_t self_raw, int8_t *xyz, uint32_t *count) {
	block::Block b;
	b.SetData(self_raw);
	const block::BlockMesh *m = b.GetCustomMesh();
	if (!m || !m->p_dynamic_mesh_func)
		return 1;
	*count = m->fetch_neighbour_count;
	for (uint32_t i = 0; i < m->fetch_neighbour_count; ++i) {
		xyz[3 * i] = m->fetch_neighbours[i].x;
		xyz[3 * i + 1] = m->fetch_neighbours[i].y;
		xyz[3 * i + 2] = m->fetch_neighbours[i].z;
	}
	return 0;
}

// ChunkShouldRemesh (client/include/client/ChunkMeshTask.inl:9-15) is the same LightAlgo's
// IsBorderLightInterfere at level 15; the .inl itself includes the renderer, so it is called here.
int hcref_chunk_should_remesh(int x, int y, int z) {
	return LightAlgo::IsBorderLightInterfere((InnerPos1)x, (InnerPos1)y, (InnerPos1)z, 15) ? 1 : 0;
}

// Same driver as the oracle's hco_mesh_many, over the reference's own templates.
uint64_t hcref_mesh_many(const uint16_t *blocks, const int8_t *heights, const int32_t *nbr, uint32_t n, int threads,
                         uint64_t *meshes_out) {
	std::atomic<uint32_t> next{0};
	std::atomic<uint64_t> quads{0}, meshes{0};
	const auto work = [&] {
		const uint16_t *b27[27];
		const int8_t *h27[27];
		Runner &r = runner();
		for (uint32_t i; (i = next.fetch_add(1)) < n;) {
			for (int k = 0; k < 27; ++k) {
				b27[k] = blocks + (size_t)nbr[(size_t)i * 27 + k] * 32768;
				h27[k] = heights + (size_t)nbr[(size_t)i * 27 + k] * 1024;
			}
			Neighbours nb{b27, h27};
			r.relight(nb);
			auto ms = r.mesh(nb);
			uint64_t q = 0;
			for (const auto &m : ms)
				q += m.vertices.size() / 4;
			quads += q;
			meshes += ms.size();
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
