// Request server: block edits, region fills, chunk loads and unloads arrive at any time and are
// batched into fixed ticks over a device-resident world.
//
// Replaces the reference's scheduling of chunk tasks: ChunkTaskPool (client/src/ChunkTaskPool.cpp:
// 16-130) queues kGenerate / kSetBlock / kSetSunlight / kMesh tasks per chunk and worker threads
// (client/src/WorldWorker.cpp:18-27) run them one chunk at a time; chunk loads arrive from
// LocalClient's loader thread (client/src/LocalClient.cpp:14-27). Here a tick thread admits, every
// tick, the requests that arrived since the last one (in arrival order, while they fit the tick's
// edit and load budgets and the pool has free slots) and enqueues one device pass for all of them:
// unloads, loads, edits, sunlight heights, then the relight + remesh of every chunk they marked. A
// completion thread waits for each pass in order, stamps its requests done and returns the pool
// slots their unloads freed. Up to `depth` passes are in flight; the copies of a pass run on their
// own stream, overlapping the compute of the passes before it.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/hc_gb300.h"
#include "hc_internal.h"

using namespace hc::detail;

namespace {

uint64_t now_ns() {
	return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
	           std::chrono::steady_clock::now().time_since_epoch())
	    .count();
}

// Waits until the steady clock reaches t (sleeps, then spins the last stretch for precision).
void wait_until_ns(uint64_t t) {
	for (;;) {
		const uint64_t n = now_ns();
		if (n >= t)
			return;
		if (t - n > 300000)
			std::this_thread::sleep_for(std::chrono::nanoseconds(t - n - 200000));
		else
			std::this_thread::yield();
	}
}

struct Pending {
	hc_request req;
	uint64_t submit_ns;
};

struct Admitted {
	uint64_t tag;
	uint32_t kind, status;
	uint64_t submit_ns;
};

constexpr uint32_t kStatusOk = 0, kStatusRejected = 1;
constexpr uint32_t kTickEntries = 1u << 20; // stored-edit entries per tick, of each kind
constexpr uint64_t kStallNs = 20000000000ull; // 20 s without a completed request

struct TickSlot {
	hc_edit *h_edits = nullptr, *d_edits = nullptr;
	int32_t *h_stage = nullptr, *d_stage = nullptr; // unload positions, load positions, load slots
	uint16_t *h_blocks = nullptr;                   // load data, pinned
	int8_t *h_heights = nullptr;
	uint32_t *h_counts = nullptr;          // pinned: world counters after the pass
	unsigned long long *h_state = nullptr; // pinned: arena cursors, work, failed
	int32_t *h_cells = nullptr;            // pinned: remesh list (when a sink is set)
	uint32_t *d_vertices = nullptr;
	uint16_t *d_indices = nullptr;
	hc_mesh_desc *d_meshes = nullptr;
	uint32_t *d_results = nullptr;
	int32_t *d_pos = nullptr;          // chunk positions of the remesh list
	hc_mesh_info *d_infos = nullptr;   // the pass's draw records
	// stored edits of the tick's loads: per load its slot and entry offsets, then the entries
	int32_t *h_dslot = nullptr, *d_dslot = nullptr;
	uint32_t *h_doff = nullptr, *d_doff = nullptr; // block offsets [L + 1], then sunlight offsets [L + 1]
	uint32_t *h_bent = nullptr, *d_bent = nullptr;
	uint16_t *h_sent = nullptr, *d_sent = nullptr;
	uint32_t n_dchunks = 0, n_bent = 0, n_sent = 0;
	cudaEvent_t start = nullptr, copied = nullptr, done = nullptr;
	uint64_t index = 0;
	std::vector<Admitted> reqs;
	std::vector<int32_t> freed;
	uint32_t n_edits = 0, n_loads = 0, n_unloads = 0;
};

} // namespace

struct hc_server {
	hc_ctx *ctx = nullptr;
	hc_pool *pool = nullptr;
	hc_world *world = nullptr;
	hc_world_desc desc{};
	hc_server_config cfg{};
	int cells = 0;
	cudaStream_t cs = nullptr, ks = nullptr, ss = nullptr; // compute, copies, sink reads
	std::vector<TickSlot> ring;
	std::vector<int32_t> cell_slot; // host mirror of the world's slots, as of the last admitted tick
	std::vector<int32_t> free_slots;

	std::mutex mu;
	std::condition_variable cv;
	std::deque<Pending> queue;
	std::deque<hc_completion> completions;
	uint64_t next_tick = 0, next_done = 0; // ticks enqueued / completed
	uint64_t submitted = 0, finished = 0;
	bool carry = false; // chunks are still marked: run the next pass even without requests
	hc_server_stats stats{};
	hc_tick_sink sink = nullptr;
	void *sink_user = nullptr;
	std::mutex step_mu; // one admitting thread at a time
	std::atomic<bool> running{false};
	std::thread tick_thread, done_thread;
	std::string err;
};

namespace {

hc_status sfail(hc_server *s, hc_status st, const std::string &m) {
	s->err = m;
	return ctx_fail(s->ctx, st, m);
}

#define SV_CUDA(s, call)                                                                                                   \
	do {                                                                                                                   \
		cudaError_t e_ = (call);                                                                                           \
		if (e_ != cudaSuccess)                                                                                             \
			return sfail(s, e_ == cudaErrorMemoryAllocation ? HC_ERR_OUT_OF_MEMORY : HC_ERR_CUDA,                          \
			             std::string(#call) + ": " + cudaGetErrorString(e_));                                              \
	} while (0)

int floor32(int v) { return v >= 0 ? v / 32 : -((-v + 31) / 32); }

int cell_of_chunk(const hc_server *s, int cx, int cy, int cz) {
	const int ix = cx - s->desc.cx0, iy = cy - s->desc.cy0, iz = cz - s->desc.cz0;
	if (ix < 0 || iy < 0 || iz < 0 || ix >= s->desc.nx || iy >= s->desc.ny || iz >= s->desc.nz)
		return -1;
	return ix + s->desc.nx * (iz + s->desc.nz * iy);
}

uint32_t fill_voxels(const hc_request &r) { return r.size * r.size * r.size; }

// Unloads a tick takes (besides max_loads_per_tick loads): an unload only drops a chunk, and a
// player's move unloads a whole shell of the view at once. Staging per tick: unload positions
// (3 x kUnloadsPerTick), then load positions (3 x L) and load slots (L).
constexpr uint32_t kUnloadsPerTick = 4096;
size_t stage_ints(uint32_t L) { return 3 * (size_t)kUnloadsPerTick + 4 * (size_t)L; }

// Decides which queued requests the next tick takes, in arrival order, stopping at the first that
// does not fit. A load or unload of a chunk that the tick already edits waits for the next tick,
// since the device pass applies unloads and loads before edits; so does a second load or unload of
// one chunk. Called with s->mu held; fills t.reqs and the host staging.
void admit(hc_server *s, TickSlot &t) {
	const hc_server_config &c = s->cfg;
	std::unordered_set<int> edited, moved;
	uint32_t ne = 0, nl = 0, nu = 0;
	t.reqs.clear();
	t.freed.clear();
	const uint32_t L = c.max_loads_per_tick;
	int32_t *unload_pos = t.h_stage;
	int32_t *load_pos = t.h_stage + 3 * kUnloadsPerTick;
	int32_t *load_slot = load_pos + 3 * L;
	t.n_dchunks = t.n_bent = t.n_sent = 0;
	t.h_doff[0] = 0, t.h_doff[L + 1] = 0;
	while (!s->queue.empty()) {
		const Pending &p = s->queue.front();
		const hc_request &r = p.req;
		uint32_t status = kStatusOk;
		if (r.kind == HC_REQ_EDIT) {
			if (ne + 1 > c.max_edits_per_tick)
				break;
			t.h_edits[ne++] = hc_edit{r.x, r.y, r.z, r.block};
			edited.insert(cell_of_chunk(s, floor32(r.x), floor32(r.y), floor32(r.z)));
		} else if (r.kind == HC_REQ_FILL) {
			const uint32_t v = fill_voxels(r);
			if (r.size == 0 || r.size > 32 || v > c.max_edits_per_tick) {
				status = kStatusRejected;
			} else {
				if (ne + v > c.max_edits_per_tick)
					break;
				for (uint32_t y = 0; y < r.size; ++y)
					for (uint32_t z = 0; z < r.size; ++z)
						for (uint32_t x = 0; x < r.size; ++x)
							t.h_edits[ne++] = hc_edit{r.x + (int)x, r.y + (int)y, r.z + (int)z, r.block};
				for (int cy = floor32(r.y); cy <= floor32(r.y + (int)r.size - 1); ++cy)
					for (int cz = floor32(r.z); cz <= floor32(r.z + (int)r.size - 1); ++cz)
						for (int cx = floor32(r.x); cx <= floor32(r.x + (int)r.size - 1); ++cx)
							edited.insert(cell_of_chunk(s, cx, cy, cz));
			}
		} else if (r.kind == HC_REQ_LOAD || r.kind == HC_REQ_UNLOAD) {
			const int cell = cell_of_chunk(s, r.x, r.y, r.z);
			const bool bad_entries = r.kind == HC_REQ_LOAD &&
			                         ((r.n_block_entries && !r.block_entries) ||
			                          (r.n_sunlight_entries && !r.sunlight_entries) ||
			                          r.n_block_entries > kTickEntries || r.n_sunlight_entries > kTickEntries);
			if (cell < 0 || (r.kind == HC_REQ_LOAD && (!r.blocks || !r.heights)) || bad_entries) {
				status = kStatusRejected;
			} else {
				if (edited.count(cell) || moved.count(cell) ||
				    (r.kind == HC_REQ_LOAD ? nl + 1 > L : nu + 1 > kUnloadsPerTick))
					break;
				if (r.kind == HC_REQ_LOAD && s->cell_slot[cell] < 0 &&
				    (t.n_bent + r.n_block_entries > kTickEntries || t.n_sent + r.n_sunlight_entries > kTickEntries))
					break; // the tick's room for stored edits is full
				if (r.kind == HC_REQ_LOAD) {
					if (s->cell_slot[cell] < 0) { // loading a resident chunk again changes nothing
						if (s->free_slots.empty())
							break; // waits for unloads to free a slot
						const int32_t slot = s->free_slots.back();
						if (r.n_block_entries || r.n_sunlight_entries) {
							const uint32_t k = t.n_dchunks++;
							t.h_dslot[k] = slot;
							if (r.n_block_entries)
								std::memcpy(t.h_bent + t.n_bent, r.block_entries, r.n_block_entries * 4);
							if (r.n_sunlight_entries)
								std::memcpy(t.h_sent + t.n_sent, r.sunlight_entries, r.n_sunlight_entries * 2);
							t.n_bent += r.n_block_entries, t.n_sent += r.n_sunlight_entries;
							t.h_doff[k + 1] = t.n_bent;
							t.h_doff[L + 1 + k + 1] = t.n_sent;
						}
						s->free_slots.pop_back();
						s->cell_slot[cell] = slot;
						std::memcpy(t.h_blocks + (size_t)nl * 32768, r.blocks, 32768 * sizeof(uint16_t));
						std::memcpy(t.h_heights + (size_t)nl * 1024, r.heights, 1024);
						load_pos[3 * nl] = r.x, load_pos[3 * nl + 1] = r.y, load_pos[3 * nl + 2] = r.z;
						load_slot[nl++] = slot;
					}
				} else if (s->cell_slot[cell] >= 0) {
					t.freed.push_back(s->cell_slot[cell]);
					s->cell_slot[cell] = -1;
					unload_pos[3 * nu] = r.x, unload_pos[3 * nu + 1] = r.y, unload_pos[3 * nu + 2] = r.z;
					++nu;
				}
				moved.insert(cell);
			}
		} else {
			status = kStatusRejected;
		}
		t.reqs.push_back(Admitted{r.tag, r.kind, status, p.submit_ns});
		s->queue.pop_front();
	}
	t.n_edits = ne, t.n_loads = nl, t.n_unloads = nu;
}

// Enqueues the device pass of tick slot t (already admitted).
hc_status enqueue_pass(hc_server *s, TickSlot &t) {
	const hc_server_config &c = s->cfg;
	const uint32_t L = c.max_loads_per_tick;
	hc_pool *pool = world_pool(s->world);
	uint16_t *pool_blocks = nullptr;
	int8_t *pool_heights = nullptr;
	hc_pool_buffers(pool, &pool_blocks, &pool_heights);
	SV_CUDA(s, cudaEventRecord(t.start, s->cs));
	// copies (own stream): edits, staged positions and slots, load data into the free slots
	if (t.n_edits)
		SV_CUDA(s, cudaMemcpyAsync(t.d_edits, t.h_edits, t.n_edits * sizeof(hc_edit), cudaMemcpyHostToDevice, s->ks));
	if (t.n_loads + t.n_unloads)
		SV_CUDA(s, cudaMemcpyAsync(t.d_stage, t.h_stage, stage_ints(L) * sizeof(int32_t), cudaMemcpyHostToDevice, s->ks));
	const int32_t *load_slot = t.h_stage + 3 * kUnloadsPerTick + 3 * L;
	for (uint32_t i = 0; i < t.n_loads; ++i) {
		SV_CUDA(s, cudaMemcpyAsync(pool_blocks + (size_t)load_slot[i] * 32768, t.h_blocks + (size_t)i * 32768,
		                           32768 * sizeof(uint16_t), cudaMemcpyHostToDevice, s->ks));
		SV_CUDA(s, cudaMemcpyAsync(pool_heights + (size_t)load_slot[i] * 1024, t.h_heights + (size_t)i * 1024, 1024,
		                           cudaMemcpyHostToDevice, s->ks));
	}
	if (t.n_dchunks) {
		SV_CUDA(s, cudaMemcpyAsync(t.d_dslot, t.h_dslot, t.n_dchunks * 4, cudaMemcpyHostToDevice, s->ks));
		SV_CUDA(s, cudaMemcpyAsync(t.d_doff, t.h_doff, 2 * (L + 1) * 4, cudaMemcpyHostToDevice, s->ks));
		if (t.n_bent)
			SV_CUDA(s, cudaMemcpyAsync(t.d_bent, t.h_bent, t.n_bent * 4, cudaMemcpyHostToDevice, s->ks));
		if (t.n_sent)
			SV_CUDA(s, cudaMemcpyAsync(t.d_sent, t.h_sent, t.n_sent * 2, cudaMemcpyHostToDevice, s->ks));
	}
	SV_CUDA(s, cudaEventRecord(t.copied, s->ks));
	SV_CUDA(s, cudaStreamWaitEvent(s->cs, t.copied, 0));
	hc_status st;
	if ((st = world_enqueue_deltas(s->world, t.d_dslot, t.d_doff, t.d_doff + L + 1, t.d_bent, t.d_sent, t.n_dchunks,
	                               s->cs)) != HC_OK ||
	    (st = world_enqueue_evict(s->world, t.d_stage, t.n_unloads, s->cs)) != HC_OK ||
	    (st = world_enqueue_place(s->world, t.d_stage + 3 * kUnloadsPerTick, t.d_stage + 3 * kUnloadsPerTick + 3 * L,
	                              t.n_loads, s->cs)) != HC_OK ||
	    (st = world_enqueue_edits(s->world, t.d_edits, t.n_edits, s->cs)) != HC_OK ||
	    (t.n_edits && (st = world_enqueue_heights(s->world, s->cs)) != HC_OK))
		return st;
	hc_batch_arena a{c.arena_quads, c.arena_meshes, t.d_vertices, t.d_indices, t.d_meshes, t.d_results};
	if ((st = world_enqueue_remesh(s->world, &a, s->cs)) != HC_OK ||
	    (st = world_enqueue_infos(s->world, &a, t.d_pos, t.d_infos, s->cs)) != HC_OK)
		return st;
	SV_CUDA(s, cudaMemcpyAsync(t.h_counts, world_counts(s->world), kWorldCountWords * sizeof(uint32_t),
	                           cudaMemcpyDeviceToHost, s->cs));
	SV_CUDA(s, cudaMemcpyAsync(t.h_state, world_state(s->world), 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
	                           s->cs));
	if (t.h_cells)
		SV_CUDA(s, cudaMemcpyAsync(t.h_cells, world_remesh_list(s->world), s->cells * sizeof(int32_t),
		                           cudaMemcpyDeviceToHost, s->cs));
	SV_CUDA(s, cudaEventRecord(t.done, s->cs));
	return HC_OK;
}

// Admits and enqueues the next tick if there is anything to do. Returns the number of requests it
// took (*ran: whether a device pass was enqueued). Waits for a free tick slot when `depth` passes
// are in flight.
hc_status start_tick(hc_server *s, uint32_t *taken, bool *ran) {
	std::lock_guard<std::mutex> step(s->step_mu);
	*taken = 0, *ran = false;
	std::unique_lock<std::mutex> lk(s->mu);
	if (!s->err.empty())
		return ctx_fail(s->ctx, HC_ERR_CUDA, s->err);
	if (s->queue.empty() && !s->carry)
		return HC_OK;
	s->cv.wait(lk, [&] { return s->next_tick - s->next_done < s->ring.size(); });
	TickSlot &t = s->ring[s->next_tick % s->ring.size()];
	if (s->sink && !t.h_cells)
		SV_CUDA(s, cudaMallocHost(&t.h_cells, s->cells * sizeof(int32_t)));
	admit(s, t);
	t.index = s->next_tick;
	*taken = (uint32_t)t.reqs.size();
	const bool work = t.n_edits || t.n_loads || t.n_unloads || s->carry;
	if (!work && t.reqs.empty())
		return HC_OK;
	s->carry = false;
	lk.unlock();
	// a tick with only rejected or no-op requests still runs, so that they complete in order
	const hc_status st = enqueue_pass(s, t);
	lk.lock();
	if (st != HC_OK)
		return st;
	++s->next_tick;
	*ran = true;
	s->cv.notify_all();
	return HC_OK;
}

// Waits for the oldest pass in flight and completes its requests. Returns false when none is.
bool finish_tick(hc_server *s, bool block) {
	TickSlot *tp;
	{
		std::unique_lock<std::mutex> lk(s->mu);
		if (block)
			s->cv.wait(lk, [&] { return s->next_done < s->next_tick || !s->running.load(); });
		if (s->next_done >= s->next_tick)
			return false;
		tp = &s->ring[s->next_done % s->ring.size()];
	}
	TickSlot &t = *tp;
	const cudaError_t ev = cudaEventSynchronize(t.done);
	const uint64_t done = now_ns();
	if (ev != cudaSuccess) { // the pass failed: stop, and report it from every later call
		std::lock_guard<std::mutex> lk(s->mu);
		s->err = std::string("device pass failed: ") + cudaGetErrorString(ev);
		s->running.store(false);
		++s->next_done;
		s->cv.notify_all();
		return true;
	}
	float ms = 0.f;
	cudaEventElapsedTime(&ms, t.start, t.done);
	const uint32_t n = t.h_counts[kWorldCountRemesh];
	const uint64_t quads = std::min<unsigned long long>(t.h_state[0], s->cfg.arena_quads);
	const uint32_t meshes = std::min<uint32_t>((uint32_t)(t.h_state[1] & 0xffffffffu), s->cfg.arena_meshes);
	const uint64_t failed = t.h_state[3];
	if (s->sink && t.h_cells) {
		// test and tooling path: the pass's output, read back before the slot is reused
		std::vector<uint32_t> res((size_t)n * 5), verts((size_t)quads * 8);
		std::vector<uint16_t> idx((size_t)quads * 6);
		std::vector<hc_mesh_desc> md(meshes);
		std::vector<hc_mesh_info> mi(meshes);
		if (n)
			cudaMemcpyAsync(res.data(), t.d_results, res.size() * 4, cudaMemcpyDeviceToHost, s->ss);
		if (quads) {
			cudaMemcpyAsync(verts.data(), t.d_vertices, verts.size() * 4, cudaMemcpyDeviceToHost, s->ss);
			cudaMemcpyAsync(idx.data(), t.d_indices, idx.size() * 2, cudaMemcpyDeviceToHost, s->ss);
		}
		if (meshes) {
			cudaMemcpyAsync(md.data(), t.d_meshes, md.size() * sizeof(hc_mesh_desc), cudaMemcpyDeviceToHost, s->ss);
			cudaMemcpyAsync(mi.data(), t.d_infos, mi.size() * sizeof(hc_mesh_info), cudaMemcpyDeviceToHost, s->ss);
		}
		cudaStreamSynchronize(s->ss);
		s->sink(s->sink_user, t.index, n, t.h_cells, res.data(), verts.data(), idx.data(), md.data(), mi.data(), quads,
		        meshes);
	}
	std::lock_guard<std::mutex> lk(s->mu);
	for (const Admitted &a : t.reqs) {
		s->completions.push_back(hc_completion{a.tag, a.kind, a.status, t.index, a.submit_ns, done});
		++s->stats.requests_done;
		if (a.status != kStatusOk)
			++s->stats.requests_rejected;
	}
	s->finished += t.reqs.size();
	for (int32_t slot : t.freed)
		s->free_slots.push_back(slot);
	s->stats.ticks += 1;
	s->stats.chunks_remeshed += n - failed;
	s->stats.quads += quads;
	s->stats.chunks_requeued += failed;
	s->stats.edits += t.n_edits;
	s->stats.loads += t.n_loads;
	s->stats.unloads += t.n_unloads;
	const uint64_t gpu = (uint64_t)(ms * 1e6);
	s->stats.gpu_ns_total += gpu;
	s->stats.gpu_ns_max = std::max<uint64_t>(s->stats.gpu_ns_max, gpu);
	s->carry = s->carry || t.h_counts[kWorldCountDirty] > 0;
	++s->next_done;
	s->cv.notify_all();
	return true;
}

void tick_loop(hc_server *s) {
	uint64_t next = now_ns();
	while (s->running.load()) {
		next += (uint64_t)s->cfg.tick_us * 1000;
		wait_until_ns(next);
		uint32_t taken;
		bool ran;
		if (start_tick(s, &taken, &ran) != HC_OK) {
			s->running.store(false);
			s->cv.notify_all();
			return;
		}
	}
}

void done_loop(hc_server *s) {
	for (;;) {
		if (!finish_tick(s, true)) {
			std::lock_guard<std::mutex> lk(s->mu);
			if (!s->running.load() && s->next_done >= s->next_tick)
				return;
		}
	}
}

void free_slot(TickSlot &t) {
	cudaFreeHost(t.h_edits);
	cudaFreeHost(t.h_stage);
	cudaFreeHost(t.h_blocks);
	cudaFreeHost(t.h_heights);
	cudaFreeHost(t.h_counts);
	cudaFreeHost(t.h_state);
	cudaFreeHost(t.h_cells);
	for (void *p : {(void *)t.h_dslot, (void *)t.h_doff, (void *)t.h_bent, (void *)t.h_sent})
		cudaFreeHost(p);
	for (void *p : {(void *)t.d_edits, (void *)t.d_stage, (void *)t.d_vertices, (void *)t.d_indices, (void *)t.d_meshes,
	                (void *)t.d_results, (void *)t.d_dslot, (void *)t.d_doff, (void *)t.d_bent, (void *)t.d_sent,
	                (void *)t.d_pos, (void *)t.d_infos})
		cudaFree(p);
	for (cudaEvent_t e : {t.start, t.copied, t.done})
		if (e)
			cudaEventDestroy(e);
}

} // namespace

extern "C" {

hc_status hc_server_create(hc_ctx *ctx, const hc_world_desc *desc, uint32_t pool_capacity,
                           const hc_server_config *config, hc_server **out) {
	if (!ctx || !desc || !config || !out || config->tick_us == 0 || config->depth == 0 || config->depth > 8 ||
	    config->max_edits_per_tick == 0 || config->max_loads_per_tick == 0 || config->arena_quads == 0 ||
	    config->arena_meshes == 0 || config->arena_quads > (1ull << 30))
		return HC_ERR_INVALID_ARG;
	const long long cells = (long long)desc->nx * desc->ny * desc->nz;
	if (desc->nx <= 0 || desc->ny <= 0 || desc->nz <= 0 || desc->ny > 32 || cells > (1ll << 21))
		return ctx_fail(ctx, HC_ERR_INVALID_ARG, "server world grid: ny <= 32 and at most 2^21 chunks");
	*out = nullptr;
	if (cudaSetDevice(ctx_device(ctx)) != cudaSuccess)
		return ctx_fail(ctx, HC_ERR_CUDA, "cudaSetDevice failed");
	hc_server *s = new hc_server();
	s->ctx = ctx, s->desc = *desc, s->cfg = *config, s->cells = (int)cells;
	const uint32_t D = config->depth, L = config->max_loads_per_tick, E = config->max_edits_per_tick;
	hc_status st = HC_OK;
	cudaError_t e = cudaSuccess;
	const auto H = [&](void **p, size_t bytes) {
		if (e == cudaSuccess)
			e = cudaMallocHost(p, bytes);
	};
	const auto A = [&](void **p, size_t bytes) {
		if (e == cudaSuccess)
			e = cudaMalloc(p, bytes);
	};
	s->ring.resize(D);
	for (TickSlot &t : s->ring) {
		H((void **)&t.h_edits, E * sizeof(hc_edit));
		A((void **)&t.d_edits, E * sizeof(hc_edit));
		H((void **)&t.h_stage, stage_ints(L) * sizeof(int32_t));
		A((void **)&t.d_stage, stage_ints(L) * sizeof(int32_t));
		H((void **)&t.h_blocks, (size_t)L * 32768 * sizeof(uint16_t));
		H((void **)&t.h_heights, (size_t)L * 1024);
		H((void **)&t.h_counts, kWorldCountWords * sizeof(uint32_t));
		H((void **)&t.h_state, 4 * sizeof(unsigned long long));
		A((void **)&t.d_vertices, config->arena_quads * 8 * sizeof(uint32_t));
		A((void **)&t.d_indices, config->arena_quads * 6 * sizeof(uint16_t) + 4);
		A((void **)&t.d_meshes, (size_t)config->arena_meshes * sizeof(hc_mesh_desc));
		A((void **)&t.d_results, (size_t)cells * 5 * sizeof(uint32_t));
		A((void **)&t.d_pos, (size_t)cells * 3 * sizeof(int32_t));
		A((void **)&t.d_infos, (size_t)config->arena_meshes * sizeof(hc_mesh_info));
		H((void **)&t.h_dslot, L * sizeof(int32_t));
		A((void **)&t.d_dslot, L * sizeof(int32_t));
		H((void **)&t.h_doff, 2 * (L + 1) * sizeof(uint32_t));
		A((void **)&t.d_doff, 2 * (L + 1) * sizeof(uint32_t));
		H((void **)&t.h_bent, kTickEntries * sizeof(uint32_t));
		A((void **)&t.d_bent, kTickEntries * sizeof(uint32_t));
		H((void **)&t.h_sent, kTickEntries * sizeof(uint16_t));
		A((void **)&t.d_sent, kTickEntries * sizeof(uint16_t));
		if (e == cudaSuccess)
			e = cudaEventCreate(&t.start);
		if (e == cudaSuccess)
			e = cudaEventCreateWithFlags(&t.copied, cudaEventDisableTiming);
		if (e == cudaSuccess)
			e = cudaEventCreate(&t.done);
		if (e == cudaSuccess)
			std::memset(t.h_stage, 0, stage_ints(L) * sizeof(int32_t));
	}
	for (cudaStream_t *q : {&s->cs, &s->ks, &s->ss})
		if (e == cudaSuccess)
			e = cudaStreamCreateWithFlags(q, cudaStreamNonBlocking);
	if (e != cudaSuccess) {
		hc_server_destroy(s);
		return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? HC_ERR_OUT_OF_MEMORY : HC_ERR_CUDA,
		                std::string("server buffers: ") + cudaGetErrorString(e));
	}
	// pool: as many slots as free device memory allows (keeping 2 GiB), at most 65536
	uint32_t cap = pool_capacity;
	if (cap == 0) {
		size_t free_b = 0, total_b = 0;
		cudaMemGetInfo(&free_b, &total_b);
		const size_t per_slot = 32768 * 2 + 1024 + pool_planes_bytes_per_slot();
		const size_t keep = (size_t)2 << 30;
		cap = (uint32_t)std::min<size_t>(65536, free_b > keep ? (free_b - keep) / per_slot : 0);
		if (cap == 0) {
			hc_server_destroy(s);
			return ctx_fail(ctx, HC_ERR_OUT_OF_MEMORY, "no device memory left for the chunk pool");
		}
	}
	if ((st = hc_pool_create(ctx, cap, &s->pool)) != HC_OK) {
		hc_server_destroy(s);
		return st;
	}
	s->cell_slot.assign(cells, -1);
	if ((st = hc_world_create(ctx, s->pool, desc, s->cell_slot.data(), &s->world)) != HC_OK ||
	    (st = hc_world_set_cluster(s->world, config->ctas_per_chunk ? (int)config->ctas_per_chunk : 4)) != HC_OK) {
		hc_server_destroy(s);
		return st;
	}
	s->free_slots.resize(cap);
	for (uint32_t i = 0; i < cap; ++i)
		s->free_slots[i] = (int32_t)(cap - 1 - i); // slot 0 is handed out first
	s->stats.pool_capacity = cap;
	*out = s;
	return HC_OK;
}

void hc_server_destroy(hc_server *s) {
	if (!s)
		return;
	hc_server_stop(s);
	cudaSetDevice(ctx_device(s->ctx));
	if (s->cs)
		cudaStreamSynchronize(s->cs);
	if (s->ks)
		cudaStreamSynchronize(s->ks);
	hc_world_destroy(s->world);
	hc_pool_destroy(s->pool);
	for (TickSlot &t : s->ring)
		free_slot(t);
	for (cudaStream_t q : {s->cs, s->ks, s->ss})
		if (q)
			cudaStreamDestroy(q);
	delete s;
}

hc_status hc_server_set_sink(hc_server *s, hc_tick_sink sink, void *user) {
	if (!s || s->running.load())
		return HC_ERR_INVALID_ARG;
	s->sink = sink, s->sink_user = user;
	return HC_OK;
}

hc_status hc_server_submit(hc_server *s, const hc_request *reqs, uint32_t n) {
	if (!s || (!reqs && n))
		return HC_ERR_INVALID_ARG;
	const uint64_t t = now_ns();
	std::lock_guard<std::mutex> lk(s->mu);
	for (uint32_t i = 0; i < n; ++i)
		s->queue.push_back(Pending{reqs[i], t});
	s->submitted += n;
	return HC_OK;
}

hc_status hc_server_start(hc_server *s) {
	if (!s || s->running.load())
		return HC_ERR_INVALID_ARG;
	s->running.store(true);
	s->done_thread = std::thread(done_loop, s);
	s->tick_thread = std::thread(tick_loop, s);
	return HC_OK;
}

hc_status hc_server_stop(hc_server *s) {
	if (!s)
		return HC_ERR_INVALID_ARG;
	bool stuck = false;
	if (s->running.load()) {
		// drain: every submitted request completes, and every marked chunk is remeshed; a queue that
		// makes no progress for kStallNs (a load waiting for a slot that no unload frees) ends it
		uint64_t last_change = now_ns(), last_finished = ~0ull;
		for (;;) {
			std::unique_lock<std::mutex> lk(s->mu);
			if (!s->running.load())
				break;
			if (s->queue.empty() && !s->carry && s->next_done == s->next_tick && s->finished == s->submitted)
				break;
			if (s->finished != last_finished)
				last_finished = s->finished, last_change = now_ns();
			else if (now_ns() - last_change > kStallNs) {
				stuck = true;
				break;
			}
			s->cv.wait_for(lk, std::chrono::milliseconds(1));
		}
		s->running.store(false);
		s->cv.notify_all();
	}
	if (s->tick_thread.joinable())
		s->tick_thread.join();
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->cv.notify_all();
	}
	if (s->done_thread.joinable())
		s->done_thread.join();
	if (!s->err.empty())
		return HC_ERR_CUDA;
	if (stuck)
		return sfail(s, HC_ERR_CAPACITY, "stopped with queued requests that made no progress (no free pool slot)");
	return HC_OK;
}

hc_status hc_server_step(hc_server *s, uint32_t *admitted) {
	if (!s || s->running.load())
		return HC_ERR_INVALID_ARG;
	uint32_t taken = 0;
	bool ran = false;
	const hc_status st = start_tick(s, &taken, &ran);
	if (st != HC_OK)
		return st;
	while (finish_tick(s, false)) {
	}
	if (admitted)
		*admitted = taken;
	if (!s->err.empty())
		return ctx_fail(s->ctx, HC_ERR_CUDA, s->err);
	return HC_OK;
}

hc_status hc_server_poll(hc_server *s, hc_completion *out, uint32_t cap, uint32_t *n) {
	if (!s || !n || (!out && cap))
		return HC_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(s->mu);
	uint32_t k = 0;
	while (k < cap && !s->completions.empty()) {
		out[k++] = s->completions.front();
		s->completions.pop_front();
	}
	*n = k;
	return HC_OK;
}

hc_status hc_server_get_stats(hc_server *s, hc_server_stats *out) {
	if (!s || !out)
		return HC_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(s->mu);
	*out = s->stats;
	out->resident = 0;
	for (int32_t v : s->cell_slot)
		out->resident += v >= 0;
	out->free_slots = (uint32_t)s->free_slots.size();
	out->queued = (uint32_t)s->queue.size();
	return HC_OK;
}

hc_status hc_server_resident(hc_server *s, int32_t *cell_slots) {
	if (!s || !cell_slots)
		return HC_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(s->mu);
	std::memcpy(cell_slots, s->cell_slot.data(), s->cell_slot.size() * sizeof(int32_t));
	return HC_OK;
}

hc_pool *hc_server_pool(hc_server *s) { return s ? s->pool : nullptr; }

hc_status hc_server_replay(hc_server *s, const hc_request *reqs, const uint64_t *arrival_ns, uint32_t n,
                           uint64_t *latency_ns, uint64_t *ticks, uint64_t *elapsed_ns) {
	if (!s || (n && (!reqs || !arrival_ns || !latency_ns)) || !s->running.load())
		return HC_ERR_INVALID_ARG;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->completions.clear();
	}
	std::vector<uint64_t> submit(n, 0);
	const uint64_t t0 = now_ns();
	uint32_t i = 0;
	while (i < n) {
		wait_until_ns(t0 + arrival_ns[i]);
		// everything due by now goes in at once
		const uint64_t now = now_ns();
		std::lock_guard<std::mutex> lk(s->mu);
		while (i < n && t0 + arrival_ns[i] <= now) {
			hc_request r = reqs[i];
			r.tag = i;
			s->queue.push_back(Pending{r, t0 + arrival_ns[i]});
			++s->submitted;
			++i;
		}
	}
	uint32_t got = 0;
	uint64_t last = t0, progress = now_ns();
	std::vector<hc_completion> buf(4096);
	while (got < n) {
		if (now_ns() - progress > kStallNs)
			return sfail(s, HC_ERR_CAPACITY, "replay: requests made no progress (no free pool slot)");
		{
			std::unique_lock<std::mutex> lk(s->mu);
			s->cv.wait_for(lk, std::chrono::milliseconds(1), [&] { return !s->completions.empty() || !s->running.load(); });
			if (s->completions.empty() && !s->running.load())
				return sfail(s, HC_ERR_CUDA, "server stopped during replay: " + s->err);
		}
		uint32_t k = 0;
		hc_server_poll(s, buf.data(), (uint32_t)buf.size(), &k);
		if (k)
			progress = now_ns();
		for (uint32_t j = 0; j < k; ++j) {
			const hc_completion &c = buf[j];
			if (c.tag < n) {
				latency_ns[c.tag] = c.done_ns - c.submit_ns;
				if (ticks)
					ticks[c.tag] = c.tick;
				last = std::max(last, c.done_ns);
				++got;
			}
		}
	}
	if (elapsed_ns)
		*elapsed_ns = last - t0;
	return HC_OK;
}

} // extern "C"
