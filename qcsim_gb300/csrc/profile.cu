// Launch timing: with profiling enabled, the engine brackets each kernel launch of a register with
// CUDA events on the register's stream and keeps (name, algorithmic bytes) per launch.  Reading the
// profile synchronises the stream and aggregates per name.  Used by the benchmark's roofline figures
// and by the cost-model timing recorder.
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "engine.cuh"

namespace qcs {
namespace {

struct Rec {
	std::string name;
	double bytes, fp_ops;
	cudaEvent_t a, b;
};

struct Prof {
	std::vector<Rec> recs;
	std::vector<cudaEvent_t> pool;
	bool open = false;
};

cudaEvent_t take(Prof* p) {
	if (!p->pool.empty()) {
		cudaEvent_t e = p->pool.back();
		p->pool.pop_back();
		return e;
	}
	cudaEvent_t e = nullptr;
	cudaEventCreate(&e);
	return e;
}

}  // namespace

void prof_begin(qcs_handle h, const char* name, double bytes, double fp_ops) {
	Prof* p = static_cast<Prof*>(h->prof);
	if (!p) return;
	Rec r{name, bytes, fp_ops, take(p), take(p)};
	cudaEventRecord(r.a, h->stream);
	p->recs.push_back(r);
	p->open = true;
}

void prof_end(qcs_handle h) {
	Prof* p = static_cast<Prof*>(h->prof);
	if (!p || !p->open) return;
	cudaEventRecord(p->recs.back().b, h->stream);
	p->open = false;
}

void prof_release(qcs_handle h) {
	Prof* p = static_cast<Prof*>(h->prof);
	if (!p) return;
	for (Rec& r : p->recs) {
		cudaEventDestroy(r.a);
		cudaEventDestroy(r.b);
	}
	for (cudaEvent_t e : p->pool) cudaEventDestroy(e);
	delete p;
	h->prof = nullptr;
}

}  // namespace qcs

extern "C" {

int qcs_profile_enable(qcs_handle h, int enable) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (enable && !h->prof) h->prof = new qcs::Prof;
	if (!enable) qcs::prof_release(h);
	return QCS_OK;
}

int qcs_profile_read(qcs_handle h, qcs_profile_entry* out, int capacity, int* count_out) {
	if (!h || !count_out || (capacity > 0 && !out)) return QCS_INVALID_ARGUMENT;
	auto* p = static_cast<qcs::Prof*>(h->prof);
	*count_out = 0;
	if (!p) return QCS_OK;
	cudaError_t e = cudaStreamSynchronize(h->stream);
	if (e != cudaSuccess) {
		h->err = std::string("profile: ") + cudaGetErrorString(e);
		return QCS_CUDA_ERROR;
	}
	struct Agg {
		uint64_t n = 0;
		double ms = 0, bytes = 0, fp_ops = 0;
	};
	std::map<std::string, Agg> agg;
	for (qcs::Rec& r : p->recs) {
		float ms = 0;
		cudaEventElapsedTime(&ms, r.a, r.b);
		Agg& a = agg[r.name];
		a.n += 1;
		a.ms += ms;
		a.bytes += r.bytes;
		a.fp_ops += r.fp_ops;
		p->pool.push_back(r.a);
		p->pool.push_back(r.b);
	}
	p->recs.clear();
	int i = 0;
	for (const auto& kv : agg) {
		if (i < capacity) {
			std::memset(&out[i], 0, sizeof(out[i]));
			std::strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
			out[i].launches = kv.second.n;
			out[i].milliseconds = kv.second.ms;
			out[i].bytes = kv.second.bytes;
			out[i].fp_ops = kv.second.fp_ops;
		}
		++i;
	}
	*count_out = i < capacity ? i : capacity;
	return QCS_OK;
}

}  // extern "C"
