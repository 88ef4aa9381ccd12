// .cw coefficient-file I/O, unpacking, contexts and error reporting.
//
// The .cw layout is the one of CoupledWaveStructure<T>::save / load
// (CoupledWaveStructure.h:7-55, 72-134):
//   u64 sizeof_T, u64 nPi, nPi records, u64 nLayers,
//   for each layer: T z, u64 nPr, nPr records, u64 nPt, nPt records
// with a record = 12 T (E0 xyz then k xyz, complex re/im interleaved).  Records are
// read and written as double (the viewer always instantiates <double>,
// sCWatterView.cpp:90); the precision field is read and ignored (:107-108) and written as 8.
// Unlike the reference loader, a truncated or inconsistent file is reported as
// SCW_ERR_FORMAT instead of producing garbage records.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <algorithm>
#include <new>

#include "scw_internal.h"

namespace scw {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

scw_status fail(scw_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

scw_status DevBuf::reserve(size_t n) {
    if (n <= bytes) return SCW_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t want = n + n / 4;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return fail(SCW_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    bytes = want;
    return SCW_OK;
}

void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

scw_status PinnedBuf::reserve(size_t n) {
    if (n <= bytes) return SCW_OK;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t want = n + n / 4;
    cudaError_t e = cudaMallocHost(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return fail(SCW_ERR_NOMEM, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    bytes = want;
    return SCW_OK;
}

void PinnedBuf::release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
}

static cudaEvent_t pool_event(scw_ctx c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

LaunchTimer::LaunchTimer(scw_ctx c, const char* n) : ctx(c), name(n) {
    if (!ctx->timing) return;
    a = pool_event(ctx);
    b = pool_event(ctx);
    cudaEventRecord(a, ctx->stream);
}

LaunchTimer::~LaunchTimer() {
    if (!a) return;
    cudaEventRecord(b, ctx->stream);
    ctx->timings.push_back(KernelTiming{name, a, b});
}

}  // namespace scw

using scw::fail;

extern "C" {

const char* scw_last_error(void) { return scw::g_last_error.c_str(); }
const char* scw_version(void) { return "scwatter_gb300 0.1 (sm_103a)"; }

// ------------------------------------------------------------------------------------
// Context
// ------------------------------------------------------------------------------------
scw_status scw_ctx_create(int device, void* stream, scw_ctx* out) {
    if (!out) return fail(SCW_ERR_ARG, "scw_ctx_create: null output");
    *out = nullptr;
    int n = 0;
    SCW_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(SCW_ERR_ARG, "scw_ctx_create: device out of range");
    SCW_ON_DEVICE(device);
    scw_ctx c = new (std::nothrow) scw_ctx_s();
    if (!c) return fail(SCW_ERR_NOMEM, "scw_ctx_create: host allocation");
    c->device = device;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) {
        delete c;
        return fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    }
    c->sm_count = prop.multiProcessorCount;
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            return fail(SCW_ERR_CUDA, cudaGetErrorString(e));
        }
        c->own_stream = true;
    }
    e = cudaEventCreateWithFlags(&c->desc_done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
        return fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = c;
    return SCW_OK;
}

scw_status scw_ctx_destroy(scw_ctx c) {
    if (!c) return SCW_OK;
    ::scw::DeviceScope dev_scope_(c->device);
    cudaStreamSynchronize(c->stream);
    c->scratch.release();
    c->desc.release();
    c->planes_out.release();
    c->sep_scratch.release();
    c->host_desc.release();
    if (c->tc_err) cudaFree(c->tc_err);
    for (auto& t : c->timings) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    for (auto e : c->event_pool) cudaEventDestroy(e);
    if (c->desc_done) cudaEventDestroy(c->desc_done);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return SCW_OK;
}

scw_status scw_ctx_synchronize(scw_ctx c) {
    if (!c) return fail(SCW_ERR_ARG, "null context");
    SCW_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (c->tc_pending_check && c->tc_err) {
        int flag = 0;
        SCW_CUDA_TRY(cudaMemcpy(&flag, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
        c->tc_pending_check = false;
        if (flag) return fail(SCW_ERR_TIMEOUT, "a tensor-core kernel's bounded mbarrier wait gave up");
    }
    return SCW_OK;
}

scw_status scw_ctx_stream(scw_ctx c, void** stream) {
    if (!c || !stream) return fail(SCW_ERR_ARG, "null argument");
    *stream = (void*)c->stream;
    return SCW_OK;
}

scw_status scw_ctx_set_timing(scw_ctx c, int on) {
    if (!c) return fail(SCW_ERR_ARG, "null context");
    c->timing = on != 0;
    return SCW_OK;
}

// Sums the recorded per-kernel times by name (after synchronising the stream) and clears
// them.  names: '\n'-separated list written to a buffer of name_bytes; ms/counts: up to max
// entries.  *n receives the number of distinct kernels.
scw_status scw_ctx_timing_report(scw_ctx c, char* names, int64_t name_bytes, double* ms, int64_t* counts,
                                 int max_entries, int* n) {
    if (!c || !n) return fail(SCW_ERR_ARG, "null argument");
    SCW_CUDA_TRY(cudaStreamSynchronize(c->stream));
    std::vector<std::string> keys;
    std::vector<double> tot;
    std::vector<int64_t> cnt;
    for (auto& t : c->timings) {
        float v = 0.f;
        cudaEventElapsedTime(&v, t.start, t.stop);
        size_t i = 0;
        while (i < keys.size() && keys[i] != t.name) i++;
        if (i == keys.size()) {
            keys.push_back(t.name);
            tot.push_back(0.0);
            cnt.push_back(0);
        }
        tot[i] += v;
        cnt[i] += 1;
        c->event_pool.push_back(t.start);
        c->event_pool.push_back(t.stop);
    }
    c->timings.clear();
    *n = (int)keys.size();
    std::string joined;
    for (size_t i = 0; i < keys.size(); i++) {
        if ((int)i < max_entries) {
            if (ms) ms[i] = tot[i];
            if (counts) counts[i] = cnt[i];
        }
        joined += keys[i];
        joined += "\n";
    }
    if (names && name_bytes > 0) {
        size_t m = std::min<size_t>((size_t)name_bytes - 1, joined.size());
        std::memcpy(names, joined.data(), m);
        names[m] = 0;
    }
    return SCW_OK;
}

scw_status scw_ctx_launch_count(scw_ctx c, int64_t* count) {
    if (!c || !count) return fail(SCW_ERR_ARG, "null argument");
    *count = c->launches;
    return SCW_OK;
}

// ------------------------------------------------------------------------------------
// .cw structure
// ------------------------------------------------------------------------------------
scw_status scw_cw_create(scw_cw* out) {
    if (!out) return fail(SCW_ERR_ARG, "null output");
    *out = new (std::nothrow) scw_cw_s();
    return *out ? SCW_OK : fail(SCW_ERR_NOMEM, "host allocation");
}

scw_status scw_cw_destroy(scw_cw cw) {
    delete cw;
    return SCW_OK;
}

static bool read_u64(std::ifstream& f, uint64_t& v) {
    f.read(reinterpret_cast<char*>(&v), sizeof(v));
    return bool(f);
}

static bool read_recs(std::ifstream& f, uint64_t n, uint64_t remaining, std::vector<double>& dst) {
    if (n > remaining / 96) return false;       // cannot fit in what is left of the file
    dst.resize(n * 12);
    if (n) f.read(reinterpret_cast<char*>(dst.data()), (std::streamsize)(n * 96));
    return bool(f);
}

scw_status scw_cw_load(const char* path, scw_cw* out) {
    if (!path || !out) return fail(SCW_ERR_ARG, "null argument");
    *out = nullptr;
    std::ifstream f(path, std::ios::in | std::ios::binary);
    if (!f) return fail(SCW_ERR_IO, std::string("cannot open ") + path);
    f.seekg(0, std::ios::end);
    uint64_t fsize = (uint64_t)f.tellg();
    f.seekg(0, std::ios::beg);
    auto remaining = [&]() -> uint64_t {
        std::streamoff p = f.tellg();
        return p < 0 ? 0 : fsize - (uint64_t)p;
    };
    scw_cw cw = new (std::nothrow) scw_cw_s();
    if (!cw) return fail(SCW_ERR_NOMEM, "host allocation");
    uint64_t nPi = 0, nL = 0;
    try {
        if (!read_u64(f, cw->sizeof_T) || !read_u64(f, nPi) || !read_recs(f, nPi, remaining(), cw->Pi) ||
            !read_u64(f, nL)) {
            delete cw;
            return fail(SCW_ERR_FORMAT, std::string("truncated .cw header or incident block: ") + path);
        }
        if (nL > remaining() / 24) {
            delete cw;
            return fail(SCW_ERR_FORMAT, "layer count exceeds file size");
        }
        cw->layers.resize(nL);
        for (uint64_t l = 0; l < nL; l++) {
            auto& L = cw->layers[l];
            uint64_t nPr = 0, nPt = 0;
            f.read(reinterpret_cast<char*>(&L.z), sizeof(double));
            if (!f || !read_u64(f, nPr) || !read_recs(f, nPr, remaining(), L.Pr) || !read_u64(f, nPt) ||
                !read_recs(f, nPt, remaining(), L.Pt)) {
                delete cw;
                return fail(SCW_ERR_FORMAT, "truncated .cw layer " + std::to_string(l));
            }
        }
    } catch (const std::bad_alloc&) {
        delete cw;
        return fail(SCW_ERR_NOMEM, "host allocation while reading .cw");
    }
    *out = cw;
    return SCW_OK;
}

scw_status scw_cw_save(scw_cw cw, const char* path) {
    if (!cw || !path) return fail(SCW_ERR_ARG, "null argument");
    std::ofstream f(path, std::ios::out | std::ios::binary);
    if (!f) return fail(SCW_ERR_IO, std::string("cannot create ") + path);
    uint64_t v = 8;
    f.write(reinterpret_cast<const char*>(&v), 8);
    v = cw->Pi.size() / 12;
    f.write(reinterpret_cast<const char*>(&v), 8);
    f.write(reinterpret_cast<const char*>(cw->Pi.data()), (std::streamsize)(cw->Pi.size() * 8));
    v = cw->layers.size();
    f.write(reinterpret_cast<const char*>(&v), 8);
    for (const auto& L : cw->layers) {
        f.write(reinterpret_cast<const char*>(&L.z), 8);
        v = L.Pr.size() / 12;
        f.write(reinterpret_cast<const char*>(&v), 8);
        f.write(reinterpret_cast<const char*>(L.Pr.data()), (std::streamsize)(L.Pr.size() * 8));
        v = L.Pt.size() / 12;
        f.write(reinterpret_cast<const char*>(&v), 8);
        f.write(reinterpret_cast<const char*>(L.Pt.data()), (std::streamsize)(L.Pt.size() * 8));
    }
    f.flush();
    if (!f) return fail(SCW_ERR_IO, std::string("write failed: ") + path);
    return SCW_OK;
}

scw_status scw_cw_set_incident(scw_cw cw, int64_t n, const double* waves) {
    if (!cw || n < 0 || (n > 0 && !waves)) return fail(SCW_ERR_ARG, "bad incident block");
    cw->Pi.assign(waves, waves + n * 12);
    return SCW_OK;
}

scw_status scw_cw_set_layer_count(scw_cw cw, int64_t n) {
    if (!cw || n < 0) return fail(SCW_ERR_ARG, "bad layer count");
    cw->layers.resize((size_t)n);
    return SCW_OK;
}

scw_status scw_cw_set_layer(scw_cw cw, int64_t l, double z, int64_t n_pr, const double* pr, int64_t n_pt,
                            const double* pt) {
    if (!cw || l < 0 || l >= (int64_t)cw->layers.size() || n_pr < 0 || n_pt < 0 || (n_pr && !pr) ||
        (n_pt && !pt))
        return fail(SCW_ERR_ARG, "bad layer arguments");
    auto& L = cw->layers[(size_t)l];
    L.z = z;
    L.Pr.assign(pr, pr + n_pr * 12);
    L.Pt.assign(pt, pt + n_pt * 12);
    return SCW_OK;
}

scw_status scw_cw_counts(scw_cw cw, int64_t* n_incident, int64_t* n_layers) {
    if (!cw) return fail(SCW_ERR_ARG, "null structure");
    if (n_incident) *n_incident = (int64_t)(cw->Pi.size() / 12);
    if (n_layers) *n_layers = (int64_t)cw->layers.size();
    return SCW_OK;
}

scw_status scw_cw_layer_counts(scw_cw cw, int64_t l, double* z, int64_t* n_pr, int64_t* n_pt) {
    if (!cw || l < 0 || l >= (int64_t)cw->layers.size()) return fail(SCW_ERR_ARG, "layer out of range");
    const auto& L = cw->layers[(size_t)l];
    if (z) *z = L.z;
    if (n_pr) *n_pr = (int64_t)(L.Pr.size() / 12);
    if (n_pt) *n_pt = (int64_t)(L.Pt.size() / 12);
    return SCW_OK;
}

scw_status scw_cw_get_incident(scw_cw cw, double* waves) {
    if (!cw || (!waves && !cw->Pi.empty())) return fail(SCW_ERR_ARG, "null argument");
    if (!cw->Pi.empty()) std::memcpy(waves, cw->Pi.data(), cw->Pi.size() * 8);
    return SCW_OK;
}

scw_status scw_cw_get_layer(scw_cw cw, int64_t l, double* pr, double* pt) {
    if (!cw || l < 0 || l >= (int64_t)cw->layers.size()) return fail(SCW_ERR_ARG, "layer out of range");
    const auto& L = cw->layers[(size_t)l];
    if (!L.Pr.empty()) {
        if (!pr) return fail(SCW_ERR_ARG, "null Pr buffer");
        std::memcpy(pr, L.Pr.data(), L.Pr.size() * 8);
    }
    if (!L.Pt.empty()) {
        if (!pt) return fail(SCW_ERR_ARG, "null Pt buffer");
        std::memcpy(pt, L.Pt.data(), L.Pt.size() * 8);
    }
    return SCW_OK;
}

// CoupledWaveStructure.h:141-147: index of the first layer whose z is <= the query,
// plus one; 0 when none is.
scw_status scw_cw_get_plane_index(scw_cw cw, double z, int64_t* index) {
    if (!cw || !index) return fail(SCW_ERR_ARG, "null argument");
    *index = 0;
    for (size_t l = 0; l < cw->layers.size(); l++) {
        if (z >= cw->layers[l].z) {
            *index = (int64_t)l + 1;
            return SCW_OK;
        }
    }
    return SCW_OK;
}

// ------------------------------------------------------------------------------------
// cw_allocate / cw_unpack (cpuEvaluator.cpp:34-102)
// ------------------------------------------------------------------------------------
scw_status scw_cw_allocate(scw_cw cw, int* layers, int64_t* total_waves) {
    if (!cw) return fail(SCW_ERR_ARG, "null structure");
    int64_t total = (int64_t)(cw->Pi.size() / 12);
    for (const auto& L : cw->layers) total += (int64_t)((L.Pr.size() + L.Pt.size()) / 12);
    if (total > std::numeric_limits<int>::max())
        return fail(SCW_ERR_UNSUPPORTED, "more waves than the int wave offsets of the reference layout can index");
    if (layers) *layers = (int)cw->layers.size();
    if (total_waves) *total_waves = total;
    return SCW_OK;
}

scw_status scw_cw_unpack(scw_cw cw, float* W, int* waves_begin, int* waves_end, float* z_layers) {
    if (!cw) return fail(SCW_ERR_ARG, "null structure");
    int layers = 0;
    int64_t total = 0;
    scw_status st = scw_cw_allocate(cw, &layers, &total);
    if (st != SCW_OK) return st;
    if ((total && !W) || !waves_begin || !waves_end || (layers && !z_layers))
        return fail(SCW_ERR_ARG, "null output buffer");
    int64_t idx = 0;
    auto copy = [&](const std::vector<double>& src) {
        for (size_t i = 0; i < src.size(); i++) W[idx * 12 + (int64_t)i] = (float)src[i];
        idx += (int64_t)(src.size() / 12);
    };
    waves_begin[0] = 0;
    copy(cw->Pi);
    for (int l = 0; l < layers; l++) {
        const auto& L = cw->layers[(size_t)l];
        z_layers[l] = (float)L.z;
        copy(L.Pr);
        waves_end[l] = (int)idx;
        waves_begin[l + 1] = (int)idx;
        copy(L.Pt);
    }
    waves_end[layers] = (int)idx;
    return SCW_OK;
}

}  // extern "C"
