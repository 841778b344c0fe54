// Serving loop: scene residency under an HBM budget (LRU eviction, rebuild
// on demand) and continuous batching of ray-batch requests from many
// sessions.  Built only on the public C ABI (lrx_scene_*, lrx_trace,
// lrx_trace_batches); declarations in include/lrx.h.
//
// Threads: callers submit and wait from any thread; one worker thread per
// server owns every CUDA call.  The worker (1) reaps finished launches by
// polling their completion events, (2) when a stream is free, takes the
// pending requests it can admit, oldest first, up to max_requests_per_launch
// requests or max_rays_per_launch rays -- making each scene resident first,
// evicting least-recently-used idle scenes while the budget is exceeded --
// and launches them together through the queue kernel (or, under the plain
// policy, one lrx_trace per request on a single stream), and (3) sleeps on a
// condition variable when there is nothing to do.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "lrx_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct SceneEntry {
	std::vector<std::vector<float>> verts;      // host copy of the geometry
	std::vector<std::vector<uint32_t>> tris;
	std::vector<lrx_mesh_desc> meshes;          // points into verts / tris
	std::vector<lrx_object_desc> objects;
	bool has_objects = false;
	uint64_t est_bytes = 0;                     // estimate until built, then exact
	bool exact = false;                         // est_bytes is a measured size
	lrx_scene *scene = nullptr;                 // resident when not null
	std::vector<unsigned char> blob;            // the built scene, kept on eviction (lrx_scene_save)
	uint64_t bytes = 0;
	uint64_t last_used = 0;
	uint32_t inflight = 0;                      // requests of this scene on the GPU
};

struct Request {
	uint64_t ticket;
	uint32_t scene;
	const void *rays;
	void *hits;
	uint32_t count, mode;
	Clock::time_point submitted;
};

struct Slot {
	cudaStream_t stream = nullptr;
	cudaEvent_t done = nullptr;
	bool busy = false;
	std::vector<Request> reqs;
	std::vector<char> fin;           // request already completed through its flag
	uint32_t *d_counters = nullptr;  // tile counters of the queue launch
	uint32_t *h_flags = nullptr;     // host-mapped completion flags, one per request
	uint32_t *d_flags = nullptr;     // their device address
};

struct TicketState {
	bool done = false;
	lrx_status status = LRX_OK;
	std::string error;
};

double percentile(std::vector<double> v, double q) {
	if (v.empty()) return 0.0;
	const size_t k = std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5));
	std::nth_element(v.begin(), v.begin() + k, v.end());
	return v[k];
}

}  // namespace

struct lrx_server {
	lrx_server_opts opts{};
	int device = 0;
	std::mutex mu;
	std::condition_variable cv_work;   // new requests or stop
	std::condition_variable cv_done;   // a ticket finished
	std::vector<std::unique_ptr<SceneEntry>> scenes;
	std::deque<Request> pending;
	std::unordered_map<uint64_t, TicketState> tickets;
	uint64_t next_ticket = 1;
	uint64_t use_clock = 0;
	std::vector<Slot> slots;
	cudaStream_t build_stream = nullptr;
	bool stop = false;
	bool started = false;
	std::string start_error;
	std::thread worker;
	// statistics (under mu)
	std::vector<double> lat_us;
	uint64_t done_req = 0, done_rays = 0, failed = 0, builds = 0, evictions = 0, launches = 0, reloads = 0;
	uint64_t cache_bytes = 0;  // blob bytes held
	uint64_t resident = 0, peak_resident = 0;
	bool any_submit = false;
	Clock::time_point first_submit, last_done;

	void run();
	void reap(std::unique_lock<std::mutex> &lk);
	bool launch_one(std::unique_lock<std::mutex> &lk);
	void finish(const Request &r, lrx_status st, const std::string &err);
	bool make_room(uint64_t need, const std::vector<uint32_t> &pinned);
	void keep_blob(SceneEntry *e);
	lrx_status make_resident(std::unique_lock<std::mutex> &lk, uint32_t id, const std::vector<uint32_t> &pinned);
};

// Records a finished request (mu held).
void lrx_server::finish(const Request &r, lrx_status st, const std::string &err) {
	const auto now = Clock::now();
	TicketState &t = tickets[r.ticket];
	t.done = true;
	t.status = st;
	t.error = err;
	if (st == LRX_OK) {
		lat_us.push_back(std::chrono::duration<double, std::micro>(now - r.submitted).count());
		++done_req;
		done_rays += r.count;
		last_done = now;
	} else {
		++failed;
	}
}

// Keeps an evicted scene's built arrays as a blob in host memory (mu held)
// so its next admission is an upload, not a build; within host_cache_bytes,
// dropping the blobs of the least recently used scenes first.  A scene that
// alone exceeds the cache is not kept.
void lrx_server::keep_blob(SceneEntry *e) {
	if (!e->blob.empty() || opts.host_cache_bytes == UINT64_MAX) return;
	size_t n = 0;
	if (lrx_scene_save(e->scene, nullptr, &n, build_stream) != LRX_OK || n > opts.host_cache_bytes) return;
	while (cache_bytes + n > opts.host_cache_bytes) {
		SceneEntry *old = nullptr;
		for (auto &p : scenes)
			if (!p->blob.empty() && (!old || p->last_used < old->last_used)) old = p.get();
		if (!old) break;
		cache_bytes -= old->blob.size();
		std::vector<unsigned char>().swap(old->blob);
	}
	try {
		e->blob.resize(n);
	} catch (const std::bad_alloc &) {
		return;
	}
	if (lrx_scene_save(e->scene, e->blob.data(), &n, build_stream) != LRX_OK) {
		std::vector<unsigned char>().swap(e->blob);
		return;
	}
	cache_bytes += e->blob.size();
}

// Evicts least-recently-used resident scenes with nothing in flight (and not
// in `pinned`) until `need` more bytes fit the budget (mu held).
bool lrx_server::make_room(uint64_t need, const std::vector<uint32_t> &pinned) {
	const uint64_t budget = opts.budget_bytes;
	while (budget && resident + need > budget) {
		SceneEntry *victim = nullptr;
		for (uint32_t i = 0; i < scenes.size(); ++i) {
			SceneEntry *e = scenes[i].get();
			if (!e->scene || e->inflight || std::find(pinned.begin(), pinned.end(), i) != pinned.end()) continue;
			if (!victim || e->last_used < victim->last_used) victim = e;
		}
		if (!victim) return false;
		keep_blob(victim);
		lrx_scene_destroy(victim->scene);
		victim->scene = nullptr;
		resident -= victim->bytes;
		victim->bytes = 0;
		++evictions;
	}
	return true;
}

// Builds scene `id` if it is not resident.  LRX_ERR_BUSY: it does not fit
// until other work finishes.  The build itself runs with mu released.
lrx_status lrx_server::make_resident(std::unique_lock<std::mutex> &lk, uint32_t id,
		const std::vector<uint32_t> &pinned) {
	SceneEntry *e = scenes[id].get();
	if (e->scene) return LRX_OK;
	const uint64_t budget = opts.budget_bytes;
	// before the first build the size is only an estimate: make room for at
	// most the whole budget and try; afterwards the exact size decides
	if (budget && e->exact && e->est_bytes > budget) return LRX_ERR_BUDGET;
	const uint64_t need = budget ? std::min(e->est_bytes, budget) : e->est_bytes;
	if (!make_room(need, pinned)) return LRX_ERR_BUSY;
	lk.unlock();
	lrx_scene *sc = nullptr;
	lrx_status rc;
	const bool reload = !e->blob.empty();
	if (reload) {
		// an evicted scene comes back from its blob: one upload, no build
		rc = lrx::scene_load_trusted(e->blob.data(), e->blob.size(), build_stream, &sc);
	} else {
		// Admission builds the plain LBVH (no treelet passes): the first
		// build is on the first request's latency.
		lrx_build_opts bo{};
		bo.struct_size = sizeof(bo);
		bo.leaf_max = 3;
		bo.treelet_passes = 0;
		rc = lrx_scene_create(e->meshes.data(), (uint32_t)e->meshes.size(),
				e->has_objects ? e->objects.data() : nullptr, (uint32_t)e->objects.size(), &bo, build_stream, &sc);
	}
	lrx_scene_info info{};
	if (rc == LRX_OK) lrx_scene_get_info(sc, &info);
	lk.lock();
	if (rc != LRX_OK) return rc;
	e->est_bytes = info.device_bytes;
	e->exact = true;
	if (budget && info.device_bytes > budget) {  // larger than the whole budget
		lrx_scene_destroy(sc);
		return LRX_ERR_BUDGET;
	}
	e->scene = sc;
	e->bytes = info.device_bytes;
	resident += e->bytes;
	peak_resident = std::max(peak_resident, resident);
	if (reload) ++reloads;
	else ++builds;
	return LRX_OK;
}

// Starts one launch on a free stream with every admissible pending request
// (one request under the plain policy).  Returns false if nothing started.
bool lrx_server::launch_one(std::unique_lock<std::mutex> &lk) {
	Slot *slot = nullptr;
	for (Slot &s : slots)
		if (!s.busy) {
			slot = &s;
			break;
		}
	if (!slot) return false;
	const bool plain = opts.policy == LRX_SERVE_PLAIN;
	const size_t max_req = plain ? 1 : opts.max_requests_per_launch;
	std::vector<Request> take;
	std::vector<uint32_t> pinned;
	std::vector<char> drop;
	// index-based: submitters may append to `pending` while a build runs unlocked
	// oldest first, until max_requests_per_launch requests or max_rays_per_launch
	// rays (at least one request)
	uint64_t take_rays = 0;
	for (size_t i = 0; i < pending.size() && take.size() < max_req &&
			(take.empty() || take_rays < opts.max_rays_per_launch); ++i) {
		drop.resize(pending.size(), 0);
		const uint32_t sid = pending[i].scene;
		const lrx_status rc = make_resident(lk, sid, pinned);
		drop.resize(pending.size(), 0);
		if (rc == LRX_OK) {
			take.push_back(pending[i]);
			take_rays += pending[i].count;
			if (std::find(pinned.begin(), pinned.end(), sid) == pinned.end()) pinned.push_back(sid);
			drop[i] = 1;
		} else if (rc == LRX_ERR_BUSY) {
			if (plain) break;  // strict FIFO
		} else {
			finish(pending[i], rc, rc == LRX_ERR_BUDGET ? "scene larger than the server budget" : lrx_last_error());
			drop[i] = 1;
		}
	}
	drop.resize(pending.size(), 0);
	if (std::find(drop.begin(), drop.end(), 1) != drop.end()) {
		std::deque<Request> keep;
		for (size_t i = 0; i < pending.size(); ++i)
			if (!drop[i]) keep.push_back(pending[i]);
		pending.swap(keep);
		cv_done.notify_all();  // some requests may have failed admission
	}
	if (take.empty()) return false;
	for (const Request &r : take) {
		scenes[r.scene]->inflight++;
		scenes[r.scene]->last_used = ++use_clock;
	}
	// shortest first: the queue kernel hands out tiles in batch order, so small
	// requests finish (and raise their flags) before the large ones
	if (!plain)
		std::stable_sort(take.begin(), take.end(), [](const Request &a, const Request &b) { return a.count < b.count; });
	std::vector<lrx_batch> batch;
	batch.reserve(take.size());
	for (const Request &r : take)
		batch.push_back(lrx_batch{scenes[r.scene]->scene, r.rays, r.hits, r.count, r.mode});
	lk.unlock();
	lrx_status rc = LRX_OK;
	if (plain) {
		for (const lrx_batch &b : batch)
			if ((rc = lrx_trace(b.scene, b.d_rays, b.d_hits, b.count, b.mode, slot->stream)) != LRX_OK) break;
	} else {
		for (size_t i = 0; i < batch.size(); ++i) reinterpret_cast<volatile uint32_t *>(slot->h_flags)[i] = 0u;
		rc = lrx_trace_batches_ex(batch.data(), (uint32_t)batch.size(), slot->stream, slot->d_counters, slot->d_flags);
	}
	std::string err = rc == LRX_OK ? std::string() : std::string(lrx_last_error());
	if (rc == LRX_OK && cudaEventRecord(slot->done, slot->stream) != cudaSuccess) {
		rc = LRX_ERR_CUDA;
		err = "cudaEventRecord failed";
	}
	if (rc != LRX_OK) cudaStreamSynchronize(slot->stream);  // leave nothing running on a failed launch
	lk.lock();
	if (rc != LRX_OK) {
		for (const Request &r : take) {
			scenes[r.scene]->inflight--;
			finish(r, rc, err);
		}
		cv_done.notify_all();
		return true;
	}
	slot->reqs.swap(take);
	slot->fin.assign(slot->reqs.size(), 0);
	slot->busy = true;
	++launches;
	return true;
}

// Completes every launch whose event has fired (mu held).
void lrx_server::reap(std::unique_lock<std::mutex> &) {
	bool any = false;
	for (Slot &s : slots) {
		if (!s.busy) continue;
		if (opts.policy != LRX_SERVE_PLAIN) {
			// requests whose batch already finished inside a running launch
			for (size_t i = 0; i < s.reqs.size(); ++i) {
				if (s.fin[i] || !reinterpret_cast<volatile uint32_t *>(s.h_flags)[i]) continue;
				s.fin[i] = 1;
				scenes[s.reqs[i].scene]->inflight--;
				finish(s.reqs[i], LRX_OK, std::string());
				any = true;
			}
		}
		const cudaError_t q = cudaEventQuery(s.done);
		if (q == cudaErrorNotReady) continue;
		const lrx_status st = q == cudaSuccess ? LRX_OK : LRX_ERR_CUDA;
		const std::string err = q == cudaSuccess ? std::string() : std::string(cudaGetErrorString(q));
		for (size_t i = 0; i < s.reqs.size(); ++i) {
			if (s.fin[i]) continue;
			const Request &r = s.reqs[i];
			scenes[r.scene]->inflight--;
			finish(r, st, err);
		}
		s.reqs.clear();
		s.busy = false;
		any = true;
	}
	if (any) cv_done.notify_all();
}

void lrx_server::run() {
	std::string err;
	if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&build_stream, cudaStreamNonBlocking) != cudaSuccess)
		err = "cannot create the server's streams";
	for (Slot &s : slots) {
		if (!err.empty()) break;
		const size_t words = opts.max_requests_per_launch;
		if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
				cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess ||
				cudaMalloc(&s.d_counters, sizeof(uint32_t) * words) != cudaSuccess ||
				cudaHostAlloc(&s.h_flags, sizeof(uint32_t) * words, cudaHostAllocMapped) != cudaSuccess ||
				cudaHostGetDevicePointer((void **)&s.d_flags, s.h_flags, 0) != cudaSuccess)
			err = "cannot create the server's streams and completion flags";
	}
	std::unique_lock<std::mutex> lk(mu);
	started = true;
	start_error = err;
	cv_done.notify_all();
	if (!err.empty()) return;
	for (;;) {
		reap(lk);
		bool busy = false;
		for (const Slot &s : slots) busy |= s.busy;
		if (stop && pending.empty() && !busy) break;
		if (!pending.empty() && launch_one(lk)) continue;
		if (busy) {  // poll the launches in flight
			lk.unlock();
			std::this_thread::yield();
			lk.lock();
			continue;
		}
		if (!pending.empty()) {  // waiting for memory that nothing in flight will free
			cv_work.wait_for(lk, std::chrono::milliseconds(1));
			continue;
		}
		cv_work.wait(lk, [&] { return stop || !pending.empty(); });
	}
	for (Slot &s : slots) {
		if (s.done) cudaEventDestroy(s.done);
		if (s.stream) cudaStreamDestroy(s.stream);
		if (s.d_counters) cudaFree(s.d_counters);
		if (s.h_flags) cudaFreeHost(s.h_flags);
	}
	if (build_stream) cudaStreamDestroy(build_stream);
}

extern "C" {

lrx_status lrx_server_create(const lrx_server_opts *opts, lrx_server **out) {
	if (!out) {
		lrx::set_error("lrx_server_create: null output");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	*out = nullptr;
	try {
		std::unique_ptr<lrx_server> s(new lrx_server());
		s->opts.struct_size = sizeof(lrx_server_opts);
		s->opts.policy = LRX_SERVE_BATCHED;
		s->opts.streams = 4;
		s->opts.max_requests_per_launch = 384;
		s->opts.host_cache_bytes = 16ull << 30;
		s->opts.max_rays_per_launch = 2ull << 20;
		if (opts) {
			if (opts->struct_size < offsetof(lrx_server_opts, host_cache_bytes) || opts->policy > LRX_SERVE_PLAIN ||
					opts->streams > 64) {
				lrx::set_error("lrx_server_create: bad options");
				return LRX_ERR_INVALID_ARGUMENT;
			}
			// fields past the caller's struct keep their defaults
			if (opts->struct_size >= offsetof(lrx_server_opts, host_cache_bytes) + sizeof(uint64_t) &&
					opts->host_cache_bytes)
				s->opts.host_cache_bytes = opts->host_cache_bytes;
			if (opts->struct_size >= offsetof(lrx_server_opts, max_rays_per_launch) + sizeof(uint64_t) &&
					opts->max_rays_per_launch)
				s->opts.max_rays_per_launch = opts->max_rays_per_launch;
			s->opts.policy = opts->policy;
			s->opts.budget_bytes = opts->budget_bytes;
			if (opts->streams) s->opts.streams = opts->streams;
			if (opts->max_requests_per_launch) s->opts.max_requests_per_launch = opts->max_requests_per_launch;
		}
		if (s->opts.policy == LRX_SERVE_PLAIN) s->opts.streams = 1;
		LRX_CUDA(cudaGetDevice(&s->device));
		s->slots.resize(s->opts.streams);
		lrx_server *raw = s.get();
		s->worker = std::thread([raw] { raw->run(); });
		std::unique_lock<std::mutex> lk(s->mu);
		s->cv_done.wait(lk, [&] { return s->started; });
		if (!s->start_error.empty()) {
			lrx::set_error(s->start_error);
			lk.unlock();
			s->worker.join();
			return LRX_ERR_CUDA;
		}
		lk.unlock();
		*out = s.release();
		return LRX_OK;
	} catch (const std::exception &e) {
		lrx::set_error(std::string("lrx_server_create: ") + e.what());
		return LRX_ERR_OUT_OF_MEMORY;
	}
}

lrx_status lrx_server_destroy(lrx_server *s) {
	if (!s) return LRX_OK;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_work.notify_all();
	if (s->worker.joinable()) s->worker.join();
	for (auto &e : s->scenes)
		if (e->scene) lrx_scene_destroy(e->scene);
	delete s;
	return LRX_OK;
}

lrx_status lrx_server_add_scene(lrx_server *s, const lrx_mesh_desc *meshes, uint32_t mesh_count,
		const lrx_object_desc *objects, uint32_t object_count, uint32_t *out_id) {
	if (!s || !out_id || (mesh_count && !meshes)) {
		lrx::set_error("lrx_server_add_scene: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	try {
		std::unique_ptr<SceneEntry> e(new SceneEntry());
		uint64_t tris = 0;
		for (uint32_t i = 0; i < mesh_count; ++i) {
			const lrx_mesh_desc &m = meshes[i];
			if ((m.vertex_count && !m.vertices) || (m.triangle_count && !m.triangles)) {
				lrx::set_error("lrx_server_add_scene: null vertex or triangle pointer");
				return LRX_ERR_INVALID_ARGUMENT;
			}
			e->verts.emplace_back(m.vertices, m.vertices + 3ull * m.vertex_count);
			e->tris.emplace_back(m.triangles, m.triangles + 3ull * m.triangle_count);
		}
		for (uint32_t i = 0; i < mesh_count; ++i)
			e->meshes.push_back(lrx_mesh_desc{e->verts[i].data(), e->tris[i].data(), meshes[i].vertex_count,
					meshes[i].triangle_count});
		if (objects) {
			e->has_objects = true;
			e->objects.assign(objects, objects + object_count);
			for (const lrx_object_desc &o : e->objects)
				if (o.mesh < mesh_count) tris += meshes[o.mesh].triangle_count;
		} else {
			for (uint32_t i = 0; i < mesh_count; ++i) tris += meshes[i].triangle_count;
		}
		// first estimate: ~13 B of wide nodes + 48 B of triangle record per
		// unique triangle, 160 B per object; replaced by the exact size once built
		uint64_t unique = 0;
		for (uint32_t i = 0; i < mesh_count; ++i) unique += meshes[i].triangle_count;
		e->est_bytes = 64ull * unique + 160ull * (objects ? object_count : mesh_count) + 4096;
		(void)tris;
		std::lock_guard<std::mutex> lk(s->mu);
		*out_id = (uint32_t)s->scenes.size();
		s->scenes.push_back(std::move(e));
		return LRX_OK;
	} catch (const std::bad_alloc &) {
		lrx::set_error("lrx_server_add_scene: host allocation failed");
		return LRX_ERR_OUT_OF_MEMORY;
	}
}

lrx_status lrx_server_submit(lrx_server *s, uint32_t scene_id, const void *d_rays, void *d_hits, uint32_t count,
		uint32_t mode, uint64_t *out_ticket) {
	if (!s || !out_ticket || mode > LRX_TRACE_ANY || (count && (!d_rays || !d_hits))) {
		lrx::set_error("lrx_server_submit: null argument or unknown mode");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (((uintptr_t)d_rays & 15u) || ((uintptr_t)d_hits & 3u)) {
		lrx::set_error("lrx_server_submit: rays must be 16-byte aligned, hits 4-byte aligned");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	{
		std::lock_guard<std::mutex> lk(s->mu);
		if (scene_id >= s->scenes.size()) {
			lrx::set_error("lrx_server_submit: unknown scene id");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		if (s->stop) {
			lrx::set_error("lrx_server_submit: server is stopping");
			return LRX_ERR_BUSY;
		}
		const auto now = Clock::now();
		if (!s->any_submit) {
			s->any_submit = true;
			s->first_submit = now;
		}
		const uint64_t t = s->next_ticket++;
		s->tickets[t] = TicketState{};
		if (count == 0) {
			s->finish(Request{t, scene_id, d_rays, d_hits, 0, mode, now}, LRX_OK, std::string());
		} else {
			s->pending.push_back(Request{t, scene_id, d_rays, d_hits, count, mode, now});
		}
		*out_ticket = t;
	}
	s->cv_work.notify_one();
	return LRX_OK;
}

lrx_status lrx_server_wait(lrx_server *s, uint64_t ticket, uint32_t timeout_ms) {
	if (!s) {
		lrx::set_error("lrx_server_wait: null server");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	std::unique_lock<std::mutex> lk(s->mu);
	auto it = s->tickets.find(ticket);
	if (it == s->tickets.end()) {
		lrx::set_error("lrx_server_wait: unknown or already collected ticket");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return s->tickets[ticket].done; }))
		return LRX_ERR_TIMEOUT;
	const TicketState st = s->tickets[ticket];
	s->tickets.erase(ticket);
	if (st.status != LRX_OK) lrx::set_error("request failed: " + st.error);
	return st.status;
}

lrx_status lrx_server_get_stats(lrx_server *s, lrx_server_stats *out) {
	if (!s || !out) {
		lrx::set_error("lrx_server_get_stats: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	std::lock_guard<std::mutex> lk(s->mu);
	lrx_server_stats r{};
	r.requests_done = s->done_req;
	r.rays_done = s->done_rays;
	r.requests_failed = s->failed;
	r.scene_builds = s->builds;
	r.scene_evictions = s->evictions;
	r.resident_bytes = s->resident;
	r.peak_resident_bytes = s->peak_resident;
	r.launches = s->launches;
	r.latency_p50_us = percentile(s->lat_us, 0.50);
	r.latency_p99_us = percentile(s->lat_us, 0.99);
	double sum = 0.0, mx = 0.0;
	for (double v : s->lat_us) {
		sum += v;
		mx = std::max(mx, v);
	}
	r.latency_mean_us = s->lat_us.empty() ? 0.0 : sum / (double)s->lat_us.size();
	r.latency_max_us = mx;
	r.busy_seconds = (s->any_submit && s->done_req)
			? std::chrono::duration<double>(s->last_done - s->first_submit).count() : 0.0;
	r.scene_reloads = s->reloads;
	r.host_cache_bytes = s->cache_bytes;
	*out = r;
	return LRX_OK;
}

lrx_status lrx_server_reset_stats(lrx_server *s) {
	if (!s) {
		lrx::set_error("lrx_server_reset_stats: null server");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	std::lock_guard<std::mutex> lk(s->mu);
	s->lat_us.clear();
	s->done_req = s->done_rays = s->failed = s->builds = s->evictions = s->launches = s->reloads = 0;
	s->peak_resident = s->resident;
	s->any_submit = false;
	return LRX_OK;
}

}  // extern "C"
