// ensemble.cu -- many independent realisations (any mix of grid sizes) as one CUDA graph, and the
// FFT tile autotuner.  No reference counterpart: the reference runs one realisation per process.
//
// Members whose configurations differ only in the seed form batched units: one pipeline run
// covers up to max_batch of them, every pass one launch over all their grids (a 128^3 pass alone
// fills a fraction of the GPU and is bound by its launch and tail latencies).  Creation runs every
// unit once on its stream (allocating the workspaces of that stream's set and uploading the
// tables), then captures the same launches into one graph: a fork from the capture stream to S
// streams, each stream running its units back to back (largest first, so the streams finish
// together), and a join.  A replay is one cudaGraphLaunch.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "context.cuh"
#include "grids.cuh"
#include "particles.cuh"

namespace mitos {

struct Unit {
    struct ic_config cfg;             // the members' configuration (the seed of the first)
    int batch = 1;
    double *acc = nullptr;            // device P(k) accumulators, batch x (3 pk_bins + 2)
    uint64_t *states = nullptr;       // device start states, batch x 4
    double *dtab = nullptr;           // device transfer rows of cfg
    int stream = 0;
};

struct Member {
    struct ic_config cfg;
    int unit = 0, index = 0;          // realisation index within the unit
};

struct Ensemble {
    std::vector<Member> m;
    std::vector<Unit> u;
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
    for (auto &u : e->u) {
        if (u.acc) cudaFree(u.acc);
        if (u.states) cudaFree(u.states);
        if (u.dtab) cudaFree(u.dtab);
    }
    for (auto s : e->streams) cudaStreamDestroy(s);
    if (e->cap) cudaStreamDestroy(e->cap);
    if (e->t0) cudaEventDestroy(e->t0);
    if (e->t1) cudaEventDestroy(e->t1);
    delete e;
}

// configurations that one batched run can cover: all fields but the seed equal
static bool same_but_seed(const struct ic_config &a, const struct ic_config &b) {
    return a.N == b.N && a.M == b.M && a.boxlen == b.boxlen && a.A_s == b.A_s && a.n_s == b.n_s &&
           a.k_pivot == b.k_pivot && a.z_ini == b.z_ini && a.index_src == b.index_src && a.method == b.method &&
           a.ma_cycles == b.ma_cycles && a.ma_tol == b.ma_tol && a.pk_bins == b.pk_bins &&
           a.pk_linear == b.pk_linear && a.precision == b.precision;
}

static bool batchable(const struct ic_config &c) {
    return c.method != MITOS_METHOD_MONGE_AMPERE && lattice_aligned(c.N, c.M, c.boxlen);
}

// run (or capture) every unit on its stream and workspace set, in the order of e->u
static int enqueue_all(Ensemble *e, bool graph) {
    int err = 0;
    for (auto &u : e->u) {
        set_stream(e->streams[u.stream]);
        set_workspace_set(1000 + u.stream);
        PipeOpts o = {u.acc, graph};
        o.batch = u.batch;
        o.states = u.states;
        o.dtab = u.dtab;
        err = pipeline_spline(&u.cfg, e->spline, nullptr, &o);
        if (err) break;
    }
    set_stream(nullptr);
    set_workspace_set(0);
    return err;
}

// members of one unit at most this many grid cells together (a 16 x 128^3 batch)
static const double UNIT_CELLS = 33554432.0;

}  // namespace mitos

using namespace mitos;

extern "C" int ic_ensemble_create_batched(struct ic_ensemble **out, const struct ic_config *cfgs, int n,
                                          const struct perturb_spline *spline, int nstreams, int max_batch) {
    if (!out || !cfgs || n < 1 || !spline || !spline->ptdat || nstreams < 1 || max_batch < 0) {
        set_error(1, "invalid ensemble arguments");
        return 1;
    }
    Ensemble *e = new Ensemble();
    e->spline = spline;
    e->m.resize(n);
    for (int i = 0; i < n; i++) e->m[i].cfg = cfgs[i];
    // units: members in input order join the first open unit of an equal configuration
    for (int i = 0; i < n; i++) {
        const struct ic_config &c = cfgs[i];
        const double cells = pow((double)c.N, 3);
        int cap = max_batch > 0 ? max_batch : std::max(1, (int)(UNIT_CELLS / cells));
        if (!batchable(c)) cap = 1;
        int k = -1;
        for (int j = 0; j < (int)e->u.size() && k < 0; j++)
            if (e->u[j].batch < cap && same_but_seed(e->u[j].cfg, c)) k = j;
        if (k < 0) {
            e->u.emplace_back();
            e->u.back().cfg = c;
            e->u.back().batch = 0;
            k = (int)e->u.size() - 1;
        }
        e->m[i].unit = k;
        e->m[i].index = e->u[k].batch++;
    }
    // longest-processing-time assignment: units by decreasing work to the least loaded stream;
    // units keep that order within each stream
    const int nu = (int)e->u.size();
    std::vector<int> order(nu);
    for (int i = 0; i < nu; i++) order[i] = i;
    auto work = [&](int i) { return pow((double)e->u[i].cfg.N, 3) * e->u[i].batch; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work(a) > work(b); });
    const int S = std::min(nstreams, nu);
    std::vector<double> load(S, 0.0);
    std::vector<int> where(nu);
    std::vector<Unit> sorted;
    for (int i : order) {
        const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        e->u[i].stream = s;
        load[s] += work(i);
        where[i] = (int)sorted.size();
        sorted.push_back(e->u[i]);
    }
    e->u = sorted;
    for (auto &m : e->m) m.unit = where[m.unit];
    int err = 0;
    e->streams.resize(S);
    for (int s = 0; s < S && !err; s++)
        if (cudaStreamCreateWithFlags(&e->streams[s], cudaStreamNonBlocking) != cudaSuccess) err = 4;
    if (!err && (cudaStreamCreateWithFlags(&e->cap, cudaStreamNonBlocking) != cudaSuccess ||
                 cudaEventCreate(&e->t0) != cudaSuccess || cudaEventCreate(&e->t1) != cudaSuccess))
        err = 4;
    const int k_size = spline->ptdat->k_size;
    for (auto &u : e->u) {
        if (err) break;
        if (cudaMalloc(&u.acc, sizeof(double) * (3 * (size_t)u.cfg.pk_bins + 2) * u.batch) != cudaSuccess ||
            cudaMalloc(&u.states, sizeof(uint64_t) * 4 * u.batch) != cudaSuccess ||
            cudaMalloc(&u.dtab, sizeof(double) * 3 * (size_t)k_size) != cudaSuccess)
            err = 5;
    }
    if (!err) {
        // start states of every realisation, in unit order
        std::vector<std::vector<uint64_t>> st(e->u.size());
        for (size_t k = 0; k < e->u.size(); k++) st[k].resize(4 * (size_t)e->u[k].batch);
        for (auto &m : e->m) seed_state(m.cfg.seed, &st[m.unit][4 * (size_t)m.index]);
        for (size_t k = 0; k < e->u.size() && !err; k++)
            if (cudaMemcpy(e->u[k].states, st[k].data(), sizeof(uint64_t) * st[k].size(), cudaMemcpyHostToDevice) !=
                cudaSuccess)
                err = 4;
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
    // 2) capture: fork to the unit streams, run, join
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
    *out = reinterpret_cast<struct ic_ensemble *>(e);
    return 0;
}

extern "C" int ic_ensemble_create(struct ic_ensemble **out, const struct ic_config *cfgs, int n,
                                  const struct perturb_spline *spline, int nstreams) {
    return ic_ensemble_create_batched(out, cfgs, n, spline, nstreams, 0);
}

extern "C" int ic_ensemble_units(const struct ic_ensemble *ens) {
    const Ensemble *e = reinterpret_cast<const Ensemble *>(ens);
    return e ? (int)e->u.size() : 0;
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
    const double *acc = e->u[m.unit].acc + (size_t)m.index * (3 * (size_t)bins + 2);
    const double *ksum;
    const long long *count;
    int err = bin_geometry(m.cfg.N, bins, m.cfg.pk_linear, m.cfg.boxlen, &ksum, &count);
    if (err) return err;
    std::vector<double> h(bins);
    MITOS_CUDA(cudaMemcpy(h.data(), acc + bins, sizeof(double) * bins, cudaMemcpyDeviceToHost));
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

// ---- FFT schedule autotuner --------------------------------------------------------------------
// Times the whole IC of cfg (pipeline launches on the library stream, CUDA events, best of three
// after one warm-up) and keeps the fastest schedule in the grid geometry, by coordinate descent
// over three knobs: the radix schedule of the length-N transforms (X and Y passes), that of the
// length-N/2 transforms (Z passes), then the tile (pencils per block of the X / Y passes, rows per
// block of the Z passes).  Radix schedules: every order of radices 8, 4, 3, 2 dividing the
// elements a thread holds, with at most one stage more than the fewest possible.

// the ordered radix schedules of length n, at most maxst stages
static void radix_schedules(int n, int E, int maxst, std::vector<std::vector<int>> &out) {
    std::vector<int> cur;
    struct Rec {
        static void go(int rem, int E, int maxst, std::vector<int> &cur, std::vector<std::vector<int>> &out) {
            if (rem == 1) {
                if (!cur.empty()) out.push_back(cur);
                return;
            }
            if ((int)cur.size() >= maxst) return;
            for (int r : {8, 4, 3, 2})
                if (E % r == 0 && rem % r == 0) {
                    cur.push_back(r);
                    go(rem / r, E, maxst, cur, out);
                    cur.pop_back();
                }
        }
    };
    Rec::go(n, E, maxst, cur, out);
}

static int min_stages(const std::vector<std::vector<int>> &c) {
    size_t m = 99;
    for (auto &v : c) m = std::min(m, v.size());
    return (int)m;
}

extern "C" int mitos_autotune(const struct ic_config *cfg, const struct perturb_spline *spline, int *best_pxy,
                              int *best_pz, double *best_ms) {
    if (!cfg || !spline) return 1;
    const GridGeom *g = geom(cfg->N, cfg->precision);
    if (!g) return 3;
    int p0, z0;
    int err = get_tiles(cfg->N, cfg->precision, &p0, &z0);
    if (err) return err;
    cudaEvent_t a, b;
    MITOS_CUDA(cudaEventCreate(&a));
    MITOS_CUDA(cudaEventCreate(&b));
    auto timed = [&](double &t) -> int {
        PipeOpts o = {nullptr, false};
        int e = pipeline_spline(cfg, spline, nullptr, &o);
        t = 1e30;
        for (int r = 0; r < 3 && !e; r++) {
            cudaEventRecord(a, stream());
            e = pipeline_spline(cfg, spline, nullptr, &o);
            cudaEventRecord(b, stream());
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            t = std::min(t, (double)ms);
        }
        return e;
    };
    int rn[MITOS_MAX_STAGES], rh[MITOS_MAX_STAGES], nn, nh;
    get_radix(cfg->N, cfg->precision, rn, &nn, rh, &nh);
    std::vector<int> bn(rn, rn + nn), bh(rh, rh + nh);
    double best = 1e30;
    err = timed(best);
    // 1. radix schedule of the length-N transforms, 2. of the length-N/2 transforms
    for (int knob = 0; knob < 2 && !err; knob++) {
        std::vector<std::vector<int>> cands;
        const int n = knob == 0 ? cfg->N : cfg->N / 2;
        radix_schedules(n, g->E, 64, cands);
        const int lim = min_stages(cands) + 1;
        for (auto &c : cands) {
            if ((int)c.size() > lim) continue;
            const std::vector<int> &tn = knob == 0 ? c : bn, &th = knob == 0 ? bh : c;
            if (set_radix(cfg->N, cfg->precision, tn.data(), (int)tn.size(), th.data(), (int)th.size())) continue;
            double t;
            err = timed(t);
            if (err) break;
            if (t < best) {
                best = t;
                (knob == 0 ? bn : bh) = c;
            }
        }
        set_radix(cfg->N, cfg->precision, bn.data(), (int)bn.size(), bh.data(), (int)bh.size());
    }
    // 3. tiles with the chosen schedules
    int bp = p0, bz = z0;
    const int cand[] = {1, 2, 4, 8, 16, 32, 64};
    for (int px : cand)
        for (int pz : cand) {
            if (err) break;
            if (set_tiles(cfg->N, cfg->precision, px, pz)) continue;
            double t;
            err = timed(t);
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

extern "C" int mitos_set_radix(int N, int precision, const int *rad_n, int stages_n, const int *rad_h,
                               int stages_h) {
    return set_radix(N, precision, rad_n, stages_n, rad_h, stages_h);
}
extern "C" int mitos_get_radix(int N, int precision, int *rad_n, int *stages_n, int *rad_h, int *stages_h) {
    if (!rad_n || !stages_n || !rad_h || !stages_h) return 1;
    return get_radix(N, precision, rad_n, stages_n, rad_h, stages_h);
}

extern "C" int mitos_set_tiles(int N, int precision, int p_xy, int p_z) { return set_tiles(N, precision, p_xy, p_z); }
extern "C" int mitos_get_tiles(int N, int precision, int *p_xy, int *p_z) {
    if (!p_xy || !p_z) return 1;
    return get_tiles(N, precision, p_xy, p_z);
}
