// Batched solve + evaluate: many samples of uneven harmonic counts, layer counts and grids,
// solved (FP64) and evaluated (separable form, complex64) by ONE CUDA-graph launch.
//
// Layout of the work:
//  * every item is planned on the host first (solve plan, separable set shape, evaluation
//    plan with its stage-1 descriptors); the sample, tables and descriptors of all items are
//    uploaded once into an input arena;
//  * items are spread over L lanes (streams) longest-processing-time first, the cost of an
//    item being Z (2MF)^3 for the solve plus its points x modes for the evaluation; each lane
//    owns one scratch arena sized for its largest item and runs its items back to back
//    (solve -> separable coefficients -> volume), so scratch is reused without allocation;
//  * the lanes are forked from one origin stream and joined back into it during a stream
//    capture, so the whole batch is one graph; scw_batch_run is one cudaGraphLaunch;
//  * results (x, gamma, status words, field volumes) live in arenas indexed per item.
// The autotuner picks the lane count (bounded by free memory) and the output-GEMM form
// (3xTF32 or split-BF16 tcgen05, or FP32 SIMT) by timing graphs of a stratified subset of the
// cheaper half of the items, and the contraction tile shape (rows per warp) by timing the
// evaluations alone of a stratified subset of all items.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <new>
#include <numeric>
#include <vector>

#include "scw_sep.h"
#include "solve_plan.h"

using scw::fail;

namespace {

struct Item {
    scw::sv::SolvePlan sp;
    scw_sep_s sep;                 // host fields; device pointers bound per lane at capture
    scw::SepEvalPlan ep;
    scw::sv::SolveIn in{};
    scw::sv::SolveOut out{};       // x, gam, status (per item)
    double *dkx = nullptr, *dky = nullptr, *dzb = nullptr;
    char* desc = nullptr;          // device stage-1 descriptors
    float* field = nullptr;        // [Nz][Ny][Nx][3] complex64
    int Nx = 0, Ny = 0, Nz = 0;
    size_t ws_bytes = 0;           // lane scratch this item needs
    double cost = 0;
};

struct Graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t nodes = 0;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        nodes = 0;
    }
};

}  // namespace

struct scw_batch_s {
    scw_ctx ctx = nullptr;
    std::vector<Item> items;
    int lanes = 0, method = 0;
    std::vector<scw_ctx> lane_ctx;
    std::vector<cudaStream_t> lane_stream;
    std::vector<char*> lane_arena;
    std::vector<size_t> lane_bytes;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    cudaStream_t origin = nullptr;
    char *d_in = nullptr, *d_out = nullptr, *d_fields = nullptr;
    Graph g;
    long long kernels = 0;
    double tune_ms = 0;
    int tuned = 0;
    std::vector<double> tune_log;  // lanes, method, contraction tile shape, ms per candidate
    int ctr_shape = 0;             // chosen contraction tile shape (scw_sep_s::ctr_shape)
    ~scw_batch_s() {
        ::scw::DeviceScope dev_scope_(ctx ? ctx->device : -1);
        g.reset();
        for (auto c : lane_ctx) scw_ctx_destroy(c);
        for (auto s : lane_stream) cudaStreamDestroy(s);
        for (auto a : lane_arena) cudaFree(a);
        for (auto e : join) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (origin) cudaStreamDestroy(origin);
        cudaFree(d_in);
        cudaFree(d_out);
        cudaFree(d_fields);
    }
};

namespace {

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// separable buffers of one item inside its lane arena: Q (complex64), kz, exterior blocks
struct SepBufs {
    float2* Q = nullptr;
    double2* kz = nullptr;
    double2* ext = nullptr;
};

void carve_sep(const scw::sv::SolvePlan& p, scw::sv::Carver& c, SepBufs& b) {
    const size_t Z = p.Z, MF = p.MF, n = p.n;
    if (!p.external) {
        b.Q = c.take<float2>(Z * 2 * 3 * MF * n);
        b.kz = c.take<double2>(Z * 2 * n + 1);
    } else {
        b.Q = nullptr;
        b.kz = c.take<double2>(1);
    }
    b.ext = c.take<double2>(12 * MF);
}

size_t lane_need(const Item& it) {
    scw::sv::Carver c;
    scw::sv::SolveWs ws{};
    scw::sv::carve_ws(it.sp, c, ws);
    SepBufs sb;
    carve_sep(it.sp, c, sb);
    c.take<char>(it.ep.scratch_bytes);
    return c.off + 256;
}

// LPT assignment of `idx` over `lanes`; returns lane per item (indexed like idx)
std::vector<int> assign_lanes(const std::vector<Item>& items, const std::vector<int>& idx, int lanes) {
    std::vector<int> order(idx);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return items[a].cost > items[b].cost; });
    std::vector<double> load(lanes, 0.0);
    std::vector<int> lane(items.size(), 0);
    for (int i : order) {
        const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        lane[i] = l;
        load[l] += items[i].cost;
    }
    return lane;
}

scw_status ensure_lanes(scw_batch b, int lanes) {
    while ((int)b->lane_ctx.size() < lanes) {
        cudaStream_t s = nullptr;
        SCW_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        b->lane_stream.push_back(s);
        scw_ctx c = nullptr;
        scw_status st = scw_ctx_create(b->ctx->device, s, &c);
        if (st != SCW_OK) return st;
        // the tensor-core error flag is allocated here, never inside a capture
        if (cudaMalloc(&c->tc_err, sizeof(int)) != cudaSuccess) return fail(SCW_ERR_NOMEM, "cudaMalloc error flag");
        SCW_CUDA_TRY(cudaMemset(c->tc_err, 0, sizeof(int)));
        b->lane_ctx.push_back(c);
        b->lane_arena.push_back(nullptr);
        b->lane_bytes.push_back(0);
        cudaEvent_t e = nullptr;
        SCW_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->join.push_back(e);
    }
    return SCW_OK;
}

// Captures the items `idx` on `lanes` lanes with output-GEMM `method` and contraction tile shape
// `ctr_shape` into graph `g`; `eval_only`: the evaluations alone (the tile-shape tuning: their
// time does not depend on the amplitude values, which are whatever the lane arenas hold)
scw_status build_graph(scw_batch b, const std::vector<int>& idx, int lanes, int method, int ctr_shape, Graph& g,
                       bool eval_only = false) {
    g.reset();
    scw_status st = ensure_lanes(b, lanes);
    if (st != SCW_OK) return st;
    const std::vector<int> lane = assign_lanes(b->items, idx, lanes);
    std::vector<size_t> need(lanes, 0);
    for (int i : idx) need[lane[i]] = std::max(need[lane[i]], b->items[i].ws_bytes);
    for (int l = 0; l < lanes; l++) {
        if (b->lane_bytes[l] < need[l]) {
            cudaFree(b->lane_arena[l]);
            b->lane_arena[l] = nullptr;
            b->lane_bytes[l] = 0;
            if (cudaMalloc(&b->lane_arena[l], need[l]) != cudaSuccess) {
                cudaGetLastError();
                return fail(SCW_ERR_NOMEM, "scw_batch: lane scratch of " + std::to_string(need[l] >> 20) + " MiB");
            }
            b->lane_bytes[l] = need[l];
        }
    }
    // items of each lane in LPT order (largest first)
    std::vector<std::vector<int>> per_lane(lanes);
    std::vector<int> order(idx);
    std::sort(order.begin(), order.end(), [&](int x, int y) { return b->items[x].cost > b->items[y].cost; });
    for (int i : order) per_lane[lane[i]].push_back(i);

    SCW_CUDA_TRY(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed));
    scw_status rec = SCW_OK;
    long long kernels = 0;
    if (cudaEventRecord(b->fork, b->origin) != cudaSuccess) rec = fail(SCW_ERR_CUDA, "event record in capture");
    for (int l = 0; l < lanes && rec == SCW_OK; l++)
        if (cudaStreamWaitEvent(b->lane_stream[l], b->fork, 0) != cudaSuccess) rec = fail(SCW_ERR_CUDA, "fork");
    for (int l = 0; l < lanes && rec == SCW_OK; l++) {
        for (int i : per_lane[l]) {
            Item& it = b->items[i];
            scw::sv::Carver c{b->lane_arena[l], 0};
            scw::sv::SolveWs ws{};
            scw::sv::carve_ws(it.sp, c, ws);
            SepBufs sb;
            carve_sep(it.sp, c, sb);
            char* scratch = c.take<char>(it.ep.scratch_bytes);
            scw::sv::SolveOut o = it.out;
            o.Q64 = nullptr;
            o.Qsep = sb.Q;
            o.sepKz = sb.kz;
            o.sepExt = sb.ext;
            if (!eval_only) rec = scw::sv::record_solve(it.sp, it.in, ws, o, b->lane_stream[l], &kernels);
            if (rec != SCW_OK) break;
            it.sep.ctx = b->lane_ctx[l];
            it.sep.dkx = it.dkx;
            it.sep.dky = it.dky;
            it.sep.dzb = it.dzb;
            it.sep.dExt = sb.ext;
            it.sep.dKz = sb.kz;
            it.sep.dQ = sb.Q;
            it.ep.method = method;
            it.sep.ctr_shape = ctr_shape;
            const long long before = b->lane_ctx[l]->launches;
            rec = scw::sep_eval_record(&it.sep, it.ep, it.desc, scratch, it.field);
            kernels += b->lane_ctx[l]->launches - before;
            if (rec != SCW_OK) break;
        }
        if (rec == SCW_OK && cudaEventRecord(b->join[l], b->lane_stream[l]) != cudaSuccess)
            rec = fail(SCW_ERR_CUDA, "join record");
        if (rec == SCW_OK && cudaStreamWaitEvent(b->origin, b->join[l], 0) != cudaSuccess)
            rec = fail(SCW_ERR_CUDA, "join wait");
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b->origin, &graph);
    if (rec != SCW_OK) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rec;
    }
    if (ce != cudaSuccess || !graph) return fail(SCW_ERR_CUDA, std::string("scw_batch capture: ") + cudaGetErrorString(ce));
    g.graph = graph;
    SCW_CUDA_TRY(cudaGraphGetNodes(graph, nullptr, &g.nodes));
    SCW_CUDA_TRY(cudaGraphInstantiate(&g.exec, graph, 0));
    b->kernels = kernels;
    return SCW_OK;
}

scw_status time_graph(scw_batch b, Graph& g, double* ms) {
    cudaEvent_t e0, e1;
    SCW_CUDA_TRY(cudaEventCreate(&e0));
    SCW_CUDA_TRY(cudaEventCreate(&e1));
    SCW_CUDA_TRY(cudaGraphLaunch(g.exec, b->origin));          // warm
    SCW_CUDA_TRY(cudaEventRecord(e0, b->origin));
    SCW_CUDA_TRY(cudaGraphLaunch(g.exec, b->origin));
    SCW_CUDA_TRY(cudaEventRecord(e1, b->origin));
    SCW_CUDA_TRY(cudaEventSynchronize(e1));
    float f = 0;
    SCW_CUDA_TRY(cudaEventElapsedTime(&f, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = f;
    return SCW_OK;
}

}  // namespace

extern "C" {

scw_status scw_batch_destroy(scw_batch b) {
    delete b;
    return SCW_OK;
}

scw_status scw_batch_create(scw_ctx ctx, const scw_batch_item* items, int count, int lanes, int method,
                            scw_batch* out) {
    if (!ctx || !items || count < 1 || !out || lanes < 0 || lanes > 64 || method < 0 || method > 3)
        return fail(SCW_ERR_ARG, "scw_batch_create: bad arguments");
    *out = nullptr;
    SCW_ON_DEVICE(ctx->device);
    std::unique_ptr<scw_batch_s> b(new (std::nothrow) scw_batch_s());
    if (!b) return fail(SCW_ERR_NOMEM, "host allocation");
    b->ctx = ctx;
    b->items.resize(count);
    // ---- plans ----
    size_t in_bytes = 0, out_bytes = 0, field_bytes = 0;
    for (int i = 0; i < count; i++) {
        const scw_batch_item& src = items[i];
        Item& it = b->items[i];
        if (!src.sample || src.Nx < 1 || src.Ny < 1 || src.Nz < 1)
            return fail(SCW_ERR_ARG, "scw_batch_create: item " + std::to_string(i) + " has no sample or an empty grid");
        scw_status st = scw::sv::plan_solve(&src.prm, src.Z, src.Y, src.X, it.sp);
        if (st != SCW_OK) return st;
        const auto& p = it.sp;
        scw_sep_s& s = it.sep;
        s.M0 = p.M0;
        s.M1 = p.M1;
        s.MF = p.MF;
        s.Z = p.Z;
        s.J = p.external ? 0 : p.n;
        s.Jp = s.J;
        s.rule = 0;
        s.kx.resize(p.M0);
        s.ky.resize(p.M1);
        for (int a = 0; a < p.M0; a++) s.kx[a] = p.Sx[(size_t)a * p.M1] * p.k;
        for (int c = 0; c < p.M1; c++) s.ky[c] = p.Sy[(size_t)c] * p.k;
        s.zb = p.zb;
        if (p.external)        // interior layers of an external-only structure sit at z = 0 with no waves
            for (int l = 1; l < p.Z; l++) s.zb[l] = 0.0;
        s.z_layers.resize(p.Z + 1);
        for (int l = 0; l <= p.Z; l++) s.z_layers[l] = (float)s.zb[l];
        it.Nx = src.Nx;
        it.Ny = src.Ny;
        it.Nz = src.Nz;
        st = scw::sep_eval_plan(&s, 0, src.x0, src.y0, src.z0, src.dx, src.dy, src.dz, src.Nx, src.Ny, src.Nz,
                                SCW_SEP_TF32X3, it.ep);
        if (st != SCW_OK) return st;
        scw::sv::Carver ci;
        scw::sv::carve_in(p, ci, it.in);
        ci.take<double>(p.M0);
        ci.take<double>(p.M1);
        ci.take<double>(p.Z + 1);
        ci.take<char>(it.ep.desc_bytes);
        in_bytes += align256(ci.off);
        scw::sv::Carver co;
        scw::sv::carve_out(p, co, it.out, false, false);
        out_bytes += align256(co.off);
        field_bytes += align256((size_t)src.Nx * src.Ny * src.Nz * 6 * sizeof(float));
        it.ws_bytes = lane_need(it);
        const double n = p.n;
        it.cost = (double)p.Z * n * n * n * 40.0 / 2.0e9 + (double)src.Nx * src.Ny * src.Nz * (3.0 * p.MF) / 1.0e12;
    }
    // ---- arenas and uploads ----
    if (cudaMalloc(&b->d_in, in_bytes) != cudaSuccess || cudaMalloc(&b->d_out, out_bytes) != cudaSuccess ||
        cudaMalloc(&b->d_fields, field_bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(SCW_ERR_NOMEM, "scw_batch_create: input / result arenas");
    }
    size_t oi = 0, oo = 0, of = 0;
    for (int i = 0; i < count; i++) {
        Item& it = b->items[i];
        const auto& p = it.sp;
        scw::sv::Carver ci{b->d_in + oi, 0};
        scw::sv::carve_in(p, ci, it.in);
        it.dkx = ci.take<double>(p.M0);
        it.dky = ci.take<double>(p.M1);
        it.dzb = ci.take<double>(p.Z + 1);
        it.desc = ci.take<char>(it.ep.desc_bytes);
        oi += align256(ci.off);
        scw::sv::Carver co{b->d_out + oo, 0};
        scw::sv::carve_out(p, co, it.out, false, false);
        oo += align256(co.off);
        it.field = (float*)(b->d_fields + of);
        of += align256((size_t)it.Nx * it.Ny * it.Nz * 6 * sizeof(float));
        scw_status st = scw::sv::upload_inputs(p, items[i].sample, it.in, ctx->stream);
        if (st != SCW_OK) return st;
        std::vector<char> desc(it.ep.desc_bytes);
        scw::sep_eval_desc(it.ep, desc.data());
        SCW_CUDA_TRY(cudaMemcpyAsync(it.dkx, it.sep.kx.data(), sizeof(double) * p.M0, cudaMemcpyHostToDevice, ctx->stream));
        SCW_CUDA_TRY(cudaMemcpyAsync(it.dky, it.sep.ky.data(), sizeof(double) * p.M1, cudaMemcpyHostToDevice, ctx->stream));
        SCW_CUDA_TRY(cudaMemcpyAsync(it.dzb, it.sep.zb.data(), sizeof(double) * (p.Z + 1), cudaMemcpyHostToDevice,
                                     ctx->stream));
        SCW_CUDA_TRY(cudaMemcpyAsync(it.desc, desc.data(), desc.size(), cudaMemcpyHostToDevice, ctx->stream));
        SCW_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    }
    SCW_CUDA_TRY(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    SCW_CUDA_TRY(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));

    // ---- autotuning on a stratified subset (every k-th item by cost, at most 8) ----
    std::vector<int> all(count);
    std::iota(all.begin(), all.end(), 0);
    size_t free_b = 0, total_b = 0;
    SCW_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    size_t max_ws = 0;
    for (const auto& it : b->items) max_ws = std::max(max_ws, it.ws_bytes);
    const int max_lanes = (int)std::max<size_t>(1, std::min<size_t>(16, (size_t)(0.8 * free_b) / std::max<size_t>(max_ws, 1)));
    const auto t0 = std::chrono::steady_clock::now();
    if (lanes == 0 || method == 0) {
        // calibration subset: 8 items spread over the cheaper half by cost, so tuning costs a
        // bounded fraction of one batch run
        std::vector<int> by_cost(all);
        std::sort(by_cost.begin(), by_cost.end(), [&](int x, int y) { return b->items[x].cost < b->items[y].cost; });
        std::vector<int> sub;
        const int pool = std::max(1, (count + 1) / 2);
        const int want = std::min(pool, 8);
        for (int j = 0; j < want; j++) sub.push_back(by_cost[(size_t)j * pool / want]);
        int best_l = lanes ? lanes : 1, best_m = method ? method : SCW_SEP_TF32X3;
        double best = 1e300;
        if (lanes == 0) {
            for (int L : {1, 2, 4, 8, 16}) {
                if (L > max_lanes || L > (int)sub.size() * 2) break;
                Graph g;
                scw_status st = build_graph(b.get(), sub, L, best_m, 0, g);
                double ms = 0;
                if (st == SCW_OK) st = time_graph(b.get(), g, &ms);
                g.reset();
                if (st != SCW_OK) return st;
                b->tune_log.insert(b->tune_log.end(), {(double)L, (double)best_m, 0.0, ms});
                b->tuned++;
                if (ms < best) {
                    best = ms;
                    best_l = L;
                }
            }
        }
        if (method == 0) {
            best = 1e300;
            for (int m : {SCW_SEP_TF32X3, SCW_SEP_BF16X3, SCW_SEP_FP32}) {
                Graph g;
                scw_status st = build_graph(b.get(), sub, best_l, m, 0, g);
                double ms = 0;
                if (st == SCW_OK) st = time_graph(b.get(), g, &ms);
                g.reset();
                if (st != SCW_OK) return st;
                b->tune_log.insert(b->tune_log.end(), {(double)best_l, (double)m, 0.0, ms});
                b->tuned++;
                if (ms < best) {
                    best = ms;
                    best_m = m;
                }
            }
        }
        lanes = best_l;
        method = best_m;
    }
    b->lanes = std::min(lanes, max_lanes);
    b->method = method;
    // contraction tile shape: the evaluations of the calibration subset alone, each shape timed
    {
        std::vector<int> by_cost(all);
        std::sort(by_cost.begin(), by_cost.end(), [&](int x, int y) { return b->items[x].cost < b->items[y].cost; });
        std::vector<int> sub;
        const int want = std::min(count, 8);
        for (int j = 0; j < want; j++) sub.push_back(by_cost[(size_t)j * count / want]);
        double best = 1e300;
        for (int shape : {0, 1}) {
            Graph g;
            const int tl = std::min(b->lanes, (int)sub.size());
            scw_status st = build_graph(b.get(), sub, tl, b->method, shape, g, true);
            // defined amplitudes and wave numbers (zeros) for the timed evaluations
            for (int l = 0; l < tl && st == SCW_OK; l++)
                if (b->lane_arena[l] && cudaMemsetAsync(b->lane_arena[l], 0, b->lane_bytes[l], b->origin) != cudaSuccess)
                    st = fail(SCW_ERR_CUDA, "scw_batch: clearing a lane arena");
            double ms = 0;
            if (st == SCW_OK) st = time_graph(b.get(), g, &ms);
            g.reset();
            if (st != SCW_OK) return st;
            b->tune_log.insert(b->tune_log.end(), {(double)b->lanes, (double)b->method, (double)shape, ms});
            b->tuned++;
            if (ms < best) {
                best = ms;
                b->ctr_shape = shape;
            }
        }
    }
    b->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    scw_status st = build_graph(b.get(), all, b->lanes, b->method, b->ctr_shape, b->g);
    if (st != SCW_OK) return st;
    // lane error flags start clear
    for (auto c : b->lane_ctx) SCW_CUDA_TRY(cudaMemset(c->tc_err, 0, sizeof(int)));
    *out = b.release();
    return SCW_OK;
}

// One graph launch on the context's stream: every item solved and evaluated.
scw_status scw_batch_run(scw_batch b) {
    if (!b || !b->g.exec) return fail(SCW_ERR_STATE, "scw_batch_run: no graph");
    SCW_ON_DEVICE(b->ctx->device);
    SCW_CUDA_TRY(cudaGraphLaunch(b->g.exec, b->ctx->stream));
    b->ctx->launches += b->kernels;
    return SCW_OK;
}

// Waits for the last run; item_status[i] = 0, SCW_ERR_NUMERIC (eigen-solver or pivots) or
// SCW_ERR_TIMEOUT (a tensor-core wait of the item's lane gave up).
scw_status scw_batch_wait(scw_batch b, int* item_status) {
    if (!b) return fail(SCW_ERR_ARG, "null batch");
    SCW_ON_DEVICE(b->ctx->device);
    SCW_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
    std::vector<int> lane_err(b->lane_ctx.size(), 0);
    for (size_t l = 0; l < b->lane_ctx.size(); l++)
        SCW_CUDA_TRY(cudaMemcpy(&lane_err[l], b->lane_ctx[l]->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
    int bad = 0;
    for (size_t i = 0; i < b->items.size(); i++) {
        const Item& it = b->items[i];
        std::vector<int> s(3 * it.sp.Z + 1);
        SCW_CUDA_TRY(cudaMemcpy(s.data(), it.out.status, sizeof(int) * s.size(), cudaMemcpyDeviceToHost));
        int v = 0;
        for (int w : s)
            if (w) v = SCW_ERR_NUMERIC;
        if (!v && it.sep.ctx) {
            for (size_t l = 0; l < b->lane_ctx.size(); l++)
                if (b->lane_ctx[l] == it.sep.ctx && lane_err[l]) v = SCW_ERR_TIMEOUT;
        }
        if (item_status) item_status[i] = v;
        bad += v != 0;
    }
    if (bad) return fail(SCW_ERR_NUMERIC, "scw_batch_wait: " + std::to_string(bad) + " item(s) failed");
    return SCW_OK;
}

// Results of item i: x (6MF complex), gamma (Z x 2MF complex), field copied to the host
// ([Nz][Ny][Nx][3] complex64); any pointer may be NULL.  field_device receives the device address.
scw_status scw_batch_get(scw_batch b, int i, double* x, double* gamma, float* field_host, float** field_device) {
    if (!b || i < 0 || i >= (int)b->items.size()) return fail(SCW_ERR_ARG, "scw_batch_get: item out of range");
    const Item& it = b->items[i];
    SCW_ON_DEVICE(b->ctx->device);
    if (x) SCW_CUDA_TRY(cudaMemcpy(x, it.out.x, sizeof(double2) * 6 * it.sp.MF, cudaMemcpyDeviceToHost));
    if (gamma)
        SCW_CUDA_TRY(cudaMemcpy(gamma, it.out.gam, sizeof(double2) * (size_t)it.sp.Z * it.sp.n, cudaMemcpyDeviceToHost));
    if (field_host)
        SCW_CUDA_TRY(cudaMemcpy(field_host, it.field, sizeof(float) * 6 * (size_t)it.Nx * it.Ny * it.Nz,
                                cudaMemcpyDeviceToHost));
    if (field_device) *field_device = it.field;
    return SCW_OK;
}

scw_status scw_batch_item_info(scw_batch b, int i, int* M0, int* M1, int* n_slices, int64_t* points_modes) {
    if (!b || i < 0 || i >= (int)b->items.size()) return fail(SCW_ERR_ARG, "scw_batch_item_info: item out of range");
    const Item& it = b->items[i];
    if (M0) *M0 = it.sp.M0;
    if (M1) *M1 = it.sp.M1;
    if (n_slices) *n_slices = it.sp.Z;
    if (points_modes) {
        // waves a point sees: 4 MF^2 inside the sample (2MF modes per harmonic per direction),
        // 2 MF above (incident + reflected) and MF below
        int64_t pm = 0;
        const int64_t MF = it.sp.MF, per_plane = (int64_t)it.Nx * it.Ny;
        for (float z : it.ep.zlist) {
            int64_t r = 0;
            for (int l = 0; l <= it.sp.Z; l++)
                if ((double)z >= (double)it.sep.z_layers[l] - 0.001) r = l + 1;
            const int64_t w = (r == 0) ? 2 * MF : (r == it.sp.Z + 1) ? MF : (it.sp.external ? 0 : 4 * MF * MF);
            pm += w * per_plane;
        }
        *points_modes = pm;
    }
    return SCW_OK;
}

// The mixed eigen-solver's record of item i (after a run): as scw_solution_eig_info.
scw_status scw_batch_item_eig(scw_batch b, int i, int* mixed, int* accepted, int* max_steps, double* max_residual,
                              int* residual_checks) {
    if (!b || i < 0 || i >= (int)b->items.size()) return fail(SCW_ERR_ARG, "scw_batch_item_eig: item out of range");
    const Item& it = b->items[i];
    const int Z = it.sp.Z;
    std::vector<int> st(2 * Z, 0);
    std::vector<double> res(Z, 0.0);
    if (it.out.eig) {
        SCW_ON_DEVICE(b->ctx->device);
        SCW_CUDA_TRY(cudaMemcpy(st.data(), it.out.eig, sizeof(int) * 2 * Z, cudaMemcpyDeviceToHost));
        SCW_CUDA_TRY(cudaMemcpy(res.data(), it.out.eig_res, sizeof(double) * Z, cudaMemcpyDeviceToHost));
    }
    const scw::sv::EigSummary e = scw::sv::eig_summary(st.data(), st.data() + Z, res.data(), it.out.eig ? Z : 0);
    if (mixed) *mixed = it.out.eig ? 1 : 0;
    if (accepted) *accepted = e.accepted;
    if (max_steps) *max_steps = e.max_steps;
    if (max_residual) *max_residual = e.max_res;
    if (residual_checks) *residual_checks = e.checks;
    return SCW_OK;
}

scw_status scw_batch_item_eig_slices(scw_batch b, int i, int* state, int* steps, double* residual) {
    if (!b || i < 0 || i >= (int)b->items.size()) return fail(SCW_ERR_ARG, "scw_batch_item_eig_slices: item out of range");
    const Item& it = b->items[i];
    if (!it.out.eig) return fail(SCW_ERR_STATE, "scw_batch_item_eig_slices: the FP64 solver ran for every slice");
    const int Z = it.sp.Z;
    SCW_ON_DEVICE(b->ctx->device);
    if (state) SCW_CUDA_TRY(cudaMemcpy(state, it.out.eig, sizeof(int) * Z, cudaMemcpyDeviceToHost));
    if (steps) SCW_CUDA_TRY(cudaMemcpy(steps, it.out.eig + Z, sizeof(int) * Z, cudaMemcpyDeviceToHost));
    if (residual) SCW_CUDA_TRY(cudaMemcpy(residual, it.out.eig_res, sizeof(double) * Z, cudaMemcpyDeviceToHost));
    return SCW_OK;
}

scw_status scw_batch_info(scw_batch b, int* lanes, int* method, int* ctr_shape, int64_t* graph_nodes, int64_t* kernels,
                          double* tune_ms, double* tune_log, int* n_tune) {
    if (!b) return fail(SCW_ERR_ARG, "null batch");
    if (lanes) *lanes = b->lanes;
    if (method) *method = b->method;
    if (ctr_shape) *ctr_shape = b->ctr_shape;
    if (graph_nodes) *graph_nodes = (int64_t)b->g.nodes;
    if (kernels) *kernels = b->kernels;
    if (tune_ms) *tune_ms = b->tune_ms;
    if (tune_log) std::memcpy(tune_log, b->tune_log.data(), sizeof(double) * b->tune_log.size());
    if (n_tune) *n_tune = b->tuned;
    return SCW_OK;
}

}  // extern "C"
