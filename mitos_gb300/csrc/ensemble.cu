// ensemble.cu -- many independent realisations (any mix of grid sizes) as one CUDA graph, and the
// FFT tile autotuner.  No reference counterpart: the reference runs one realisation per process.
//
// Creation runs every realisation once on its stream (allocating the workspaces of that stream's
// set and uploading the tables), then captures the same launches into one graph: a fork from the
// capture stream to S streams, each stream running its realisations back to back (largest grids
// first, so the streams finish together), and a join.  A replay is one cudaGraphLaunch.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "context.cuh"
#include "grids.cuh"

namespace mitos {

struct Member {
    struct ic_config cfg;
    double *acc = nullptr;  // device P(k) accumulators
    int stream = 0;
};

struct Ensemble {
    std::vector<Member> m;
    std::vector<cudaStream_t> streams;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    const struct perturb_spline *spline = nullptr;
    long launches = 0;  // kernel launches in one replay
};

static void destroy(Ensemble *e) {
    if (!e) return;
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    for (auto &m : e->m)
        if (m.acc) cudaFree(m.acc);
    for (auto s : e->streams) cudaStreamDestroy(s);
    if (e->cap) cudaStreamDestroy(e->cap);
    if (e->t0) cudaEventDestroy(e->t0);
    if (e->t1) cudaEventDestroy(e->t1);
    delete e;
}

// run (or capture) every member on its stream and workspace set
static int enqueue_all(Ensemble *e, bool graph) {
    int err = 0;
    for (auto &m : e->m) {
        set_stream(e->streams[m.stream]);
        set_workspace_set(1000 + m.stream);
        PipeOpts o = {m.acc, graph};
        err = pipeline_spline(&m.cfg, e->spline, nullptr, &o);
        if (err) break;
    }
    set_stream(nullptr);
    set_workspace_set(0);
    return err;
}

}  // namespace mitos

using namespace mitos;

extern "C" int ic_ensemble_create(struct ic_ensemble **out, const struct ic_config *cfgs, int n,
                                  const struct perturb_spline *spline, int nstreams) {
    if (!out || !cfgs || n < 1 || !spline || nstreams < 1) {
        set_error(1, "invalid ensemble arguments");
        return 1;
    }
    Ensemble *e = new Ensemble();
    e->spline = spline;
    e->m.resize(n);
    for (int i = 0; i < n; i++) e->m[i].cfg = cfgs[i];
    // longest-processing-time assignment: members by decreasing N^3 to the least loaded stream
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cfgs[a].N > cfgs[b].N; });
    const int S = std::min(nstreams, n);
    std::vector<double> load(S, 0.0);
    for (int i : order) {
        const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        e->m[i].stream = s;
        load[s] += pow((double)cfgs[i].N, 3);
    }
    // members run in the order above within each stream
    std::vector<Member> sorted;
    for (int i : order) sorted.push_back(e->m[i]);
    std::vector<int> where(n);
    for (int k = 0; k < n; k++) where[order[k]] = k;
    e->m = sorted;
    int err = 0;
    e->streams.resize(S);
    for (int s = 0; s < S && !err; s++)
        if (cudaStreamCreateWithFlags(&e->streams[s], cudaStreamNonBlocking) != cudaSuccess) err = 4;
    if (!err && (cudaStreamCreateWithFlags(&e->cap, cudaStreamNonBlocking) != cudaSuccess ||
                 cudaEventCreate(&e->t0) != cudaSuccess || cudaEventCreate(&e->t1) != cudaSuccess))
        err = 4;
    for (auto &m : e->m) {
        if (err) break;
        if (cudaMalloc(&m.acc, sizeof(double) * (3 * (size_t)m.cfg.pk_bins + 2)) != cudaSuccess) err = 5;
    }
    if (err) {
        cudaGetLastError();
        set_error(err, "ensemble resources");
        destroy(e);
        return err;
    }
    // 1) one uncaptured pass: workspaces, tables, kernel attributes
    err = enqueue_all(e, false);
    if (!err && cudaDeviceSynchronize() != cudaSuccess) err = check_cuda(cudaGetLastError(), "ensemble warm-up");
    // 2) capture: fork to the member streams, run, join
    if (!err) {
        std::vector<cudaEvent_t> ev(S + 1);
        for (auto &x : ev) cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
        const long l0 = mitos_launch_count();
        cudaError_t ce = cudaStreamBeginCapture(e->cap, cudaStreamCaptureModeThreadLocal);
        if (ce == cudaSuccess) {
            cudaEventRecord(ev[S], e->cap);
            for (int s = 0; s < S; s++) cudaStreamWaitEvent(e->streams[s], ev[S], 0);
            err = enqueue_all(e, true);
            for (int s = 0; s < S; s++) {
                cudaEventRecord(ev[s], e->streams[s]);
                cudaStreamWaitEvent(e->cap, ev[s], 0);
            }
            ce = cudaStreamEndCapture(e->cap, &e->graph);
        }
        e->launches = mitos_launch_count() - l0;
        if (!err && ce == cudaSuccess) ce = cudaGraphInstantiate(&e->exec, e->graph, 0);
        if (!err && ce != cudaSuccess) err = check_cuda(ce, "ensemble graph capture");
        for (auto &x : ev) cudaEventDestroy(x);
    }
    if (err) {
        cudaGetLastError();
        destroy(e);
        return err;
    }
    // the caller's index i refers to cfgs[i]: keep the permutation in the member order
    std::vector<Member> back(n);
    for (int i = 0; i < n; i++) back[i] = e->m[where[i]];
    e->m = back;
    *out = reinterpret_cast<struct ic_ensemble *>(e);
    return 0;
}

extern "C" int ic_ensemble_run(struct ic_ensemble *ens, double *ms) {
    Ensemble *e = reinterpret_cast<Ensemble *>(ens);
    if (!e || !e->exec) return 1;
    MITOS_CUDA(cudaEventRecord(e->t0, e->cap));
    MITOS_CUDA(cudaGraphLaunch(e->exec, e->cap));
    MITOS_CUDA(cudaEventRecord(e->t1, e->cap));
    MITOS_CUDA(cudaEventSynchronize(e->t1));
    float t = 0;
    MITOS_CUDA(cudaEventElapsedTime(&t, e->t0, e->t1));
    if (ms) *ms = t;
    count_launch((int)e->launches);
    return 0;
}

extern "C" int ic_ensemble_result(struct ic_ensemble *ens, int i, struct ic_result *res) {
    Ensemble *e = reinterpret_cast<Ensemble *>(ens);
    if (!e || i < 0 || i >= (int)e->m.size() || !res) return 1;
    const Member &m = e->m[i];
    const int bins = m.cfg.pk_bins;
    const double *ksum;
    const long long *count;
    int err = bin_geometry(m.cfg.N, bins, m.cfg.pk_linear, m.cfg.boxlen, &ksum, &count);
    if (err) return err;
    std::vector<double> h(bins);
    MITOS_CUDA(cudaMemcpy(h.data(), m.acc + bins, sizeof(double) * bins, cudaMemcpyDeviceToHost));
    const double V = m.cfg.boxlen * m.cfg.boxlen * m.cfg.boxlen;
    for (int b = 0; b < bins; b++) {
        const double nb = (double)count[b];
        if (res->pk_obs) res->pk_obs[b] = (long)count[b];
        if (res->pk_k) res->pk_k[b] = ksum[b] / nb;
        if (res->pk_p) res->pk_p[b] = h[b] / nb / V;
    }
    res->ma_iterations = 0;
    res->ma_residual = 0;
    return 0;
}

extern "C" int ic_ensemble_launches(const struct ic_ensemble *ens) {
    const Ensemble *e = reinterpret_cast<const Ensemble *>(ens);
    return e ? (int)e->launches : 0;
}

extern "C" int ic_ensemble_destroy(struct ic_ensemble *ens) {
    destroy(reinterpret_cast<Ensemble *>(ens));
    return 0;
}

// ---- FFT tile autotuner ------------------------------------------------------------------------
// Times the whole IC of cfg (pipeline launches on the library stream, CUDA events, best of three
// after one warm-up) for each candidate tile and keeps the fastest in the grid geometry.
extern "C" int mitos_autotune(const struct ic_config *cfg, const struct perturb_spline *spline, int *best_pxy,
                              int *best_pz, double *best_ms) {
    if (!cfg || !spline) return 1;
    int p0, z0;
    int err = get_tiles(cfg->N, cfg->precision, &p0, &z0);
    if (err) return err;
    cudaEvent_t a, b;
    MITOS_CUDA(cudaEventCreate(&a));
    MITOS_CUDA(cudaEventCreate(&b));
    double best = 1e30;
    int bp = p0, bz = z0;
    const int cand[] = {1, 2, 4, 8, 16, 32, 64};
    for (int px : cand)
        for (int pz : cand) {
            if (set_tiles(cfg->N, cfg->precision, px, pz)) continue;
            PipeOpts o = {nullptr, false};
            err = pipeline_spline(cfg, spline, nullptr, &o);
            if (err) break;
            double t = 1e30;
            for (int r = 0; r < 3 && !err; r++) {
                cudaEventRecord(a, stream());
                err = pipeline_spline(cfg, spline, nullptr, &o);
                cudaEventRecord(b, stream());
                cudaEventSynchronize(b);
                float ms = 0;
                cudaEventElapsedTime(&ms, a, b);
                t = std::min(t, (double)ms);
            }
            if (err) break;
            if (t < best) {
                best = t;
                bp = px;
                bz = pz;
            }
        }
    cudaGetLastError();  // a rejected candidate leaves set_error text only
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    set_tiles(cfg->N, cfg->precision, bp, bz);
    if (err) return err;
    if (best_pxy) *best_pxy = bp;
    if (best_pz) *best_pz = bz;
    if (best_ms) *best_ms = best;
    return 0;
}

extern "C" int mitos_set_tiles(int N, int precision, int p_xy, int p_z) { return set_tiles(N, precision, p_xy, p_z); }
extern "C" int mitos_get_tiles(int N, int precision, int *p_xy, int *p_z) {
    if (!p_xy || !p_z) return 1;
    return get_tiles(N, precision, p_xy, p_z);
}
