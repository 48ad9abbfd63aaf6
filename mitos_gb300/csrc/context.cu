// context.cu -- error state, the library stream, cached per-size geometry (FFT plans, twiddle,
// window and bin tables) and the device workspace.
#include <math.h>
#include <stdarg.h>
#include <string.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "context.cuh"

namespace mitos {

static char g_err[512];
static std::mutex g_mu;
static cudaStream_t g_stream = nullptr;
static long g_launches = 0;

void set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    int n = snprintf(g_err, sizeof g_err, "[%d] ", code);
    vsnprintf(g_err + n, sizeof g_err - n, fmt, ap);
    va_end(ap);
}

int check_cuda(cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation) {
        set_error(5, "out of device memory in %s", what);
        cudaGetLastError();
        return 5;
    }
    set_error(4, "CUDA error in %s: %s", what, cudaGetErrorString(e));
    return 4;
}

// the stream every launch goes to: the library stream, or the stream a caller on this thread
// selected (set_stream; the ensemble runs each realisation on its own stream)
static thread_local cudaStream_t t_stream = nullptr;
static thread_local int t_ws_set = 0;

static int g_stream_dev = -1;
cudaStream_t stream() {
    if (t_stream) return t_stream;
    if (!g_stream) {
        cudaGetDevice(&g_stream_dev);
        cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
    }
    return g_stream;
}
int library_device() {
    stream();
    return g_stream_dev;
}
void set_stream(cudaStream_t s) { t_stream = s; }
static thread_local bool t_async = false;
void set_async(bool on) { t_async = on; }
bool async_mode() { return t_async; }
void set_workspace_set(int s) { t_ws_set = s; }

// optional per-launch timing: events recorded on the library stream around every launch
static bool g_ktime = false;
static std::vector<std::pair<const char *, std::pair<cudaEvent_t, cudaEvent_t>>> g_kev;
static cudaEvent_t g_kprev = nullptr;
static const char *g_kname = nullptr;

void launch_begin(const char *name) {
    if (!g_ktime) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, stream());
    g_kprev = e;
    g_kname = name;
}

void count_launch(int n) {
    g_launches += n;
    if (g_ktime && g_kprev) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, stream());
        g_kev.push_back({g_kname, {g_kprev, e}});
        g_kprev = nullptr;
    }
}

// the plan of length n for the radices rad[0 .. ns-1] (first stage first): each radix one of 2, 3,
// 4, 8 dividing E (a thread holds E elements: E / R butterflies a stage), their product n
bool plan_from_radices(int n, int E, int tw_len, const int *rad, int ns, FFTPlan *pl) {
    if (n < E || n % E || ns < 1 || ns >= MITOS_MAX_STAGES) return false;
    long prod = 1;
    for (int i = 0; i < ns; i++) {
        const int r = rad[i];
        if ((r != 2 && r != 3 && r != 4 && r != 8) || E % r) return false;
        prod *= r;
    }
    if (prod != n) return false;
    pl->n = n;
    pl->nst = ns;
    pl->tw_scale = tw_len / n;
    pl->twst = nullptr;
    pl->twst16 = nullptr;
    int Ns = 1;
    for (int i = 0; i < ns; i++) {
        pl->rad[i] = rad[i];
        int lg = -1;
        for (int b = 0; b < 31; b++)
            if ((1 << b) == Ns) lg = b;
        pl->lgNs[i] = lg;
        pl->twstep[i] = n / (Ns * rad[i]) * pl->tw_scale;
        Ns *= rad[i];
    }
    return true;
}

// the default schedule: radix 8 stages first (when E allows), then 4, 2 and 3
bool make_plan(int n, int E, int tw_len, FFTPlan *pl) {
    if (n < E || n % E) return false;
    int rem = n, ns = 0;
    int rad[MITOS_MAX_STAGES];
    auto push = [&](int r) { if (ns < MITOS_MAX_STAGES) rad[ns++] = r; };
    if (E % 8 == 0) {
        while (rem % 8 == 0) { push(8); rem /= 8; }
    }
    while (rem % 4 == 0 && E % 4 == 0) { push(4); rem /= 4; }
    while (rem % 2 == 0 && E % 2 == 0) { push(2); rem /= 2; }
    while (rem % 3 == 0 && E % 3 == 0) { push(3); rem /= 3; }
    if (rem != 1 || ns == 0 || ns >= MITOS_MAX_STAGES) return false;
    return plan_from_radices(n, E, tw_len, rad, ns, pl);
}

static int elems_for(int N) {
    int m = N;
    while (m % 2 == 0) m /= 2;
    if (m == 1) return 8;
    if (m == 3) return 12;
    return 0;
}

struct GeomEntry {
    GridGeom g;
    void *tw = nullptr;
    void *twst[2] = {nullptr, nullptr};  // the stage twiddle tables of plN and plH
    void *twst16 = nullptr;              // plN's for the 16-element schedule
};

// the stage table of a plan (FFTPlan::twst) from the double twiddle table tw (length N, of the
// grid), in the grid's precision: the values the table twN holds, regrouped per stage and butterfly
static void *stage_twiddles(const FFTPlan &pl, const std::vector<double> &tw, int precision) {
    std::vector<double> st;
    int Ns = pl.rad[0];
    for (int s = 1; s < pl.nst; s++) {
        const int R = pl.rad[s], TR = tw_row(R);
        for (int jm = 0; jm < Ns; jm++)
            for (int k = 0; k < TR; k++) {
                const int r = k + 1;
                const long idx = r < R ? (long)r * jm * (pl.n / (Ns * R)) * pl.tw_scale : 0;
                st.push_back(r < R ? tw[2 * idx] : 0.0);
                st.push_back(r < R ? tw[2 * idx + 1] : 0.0);
            }
        Ns *= R;
    }
    if (st.empty()) st.assign(4, 0.0);
    void *d = nullptr;
    if (precision == MITOS_FP32) {
        std::vector<float> f(st.begin(), st.end());
        if (cudaMalloc(&d, sizeof(float) * f.size()) != cudaSuccess) return nullptr;
        cudaMemcpy(d, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice);
    } else {
        if (cudaMalloc(&d, sizeof(double) * st.size()) != cudaSuccess) return nullptr;
        cudaMemcpy(d, st.data(), sizeof(double) * st.size(), cudaMemcpyHostToDevice);
    }
    return d;
}
static std::map<std::pair<int, int>, GeomEntry *> g_geoms;

const GridGeom *geom(int N, int precision) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_pair(N, precision);
    auto it = g_geoms.find(key);
    if (it != g_geoms.end()) return &it->second->g;
    int E = elems_for(N);
    if (N < 16 || N > 4096 || E == 0 || (N / 2) % E) {
        set_error(3, "grid size N = %d is not supported (2^k or 3*2^k, 16 <= N <= 4096)", N);
        return nullptr;
    }
    GeomEntry *ge = new GeomEntry;
    GridGeom &g = ge->g;
    g.N = N;
    g.H = N / 2 + 1;
    g.plane = (long)N * g.H;
    g.cells = (long)N * g.plane;
    g.E = E;
    g.custom_radix = 0;
    if (!make_plan(N, E, N, &g.plN) || !make_plan(N / 2, E, N, &g.plH)) {
        delete ge;
        set_error(3, "no FFT schedule for N = %d", N);
        return nullptr;
    }
    int tpp = N / E;
    int P = 512 / tpp;
    if (P < 1) P = 1;
    if (P > 64) P = 64;
    const size_t csz = precision == MITOS_FP32 ? 8 : 16;
    while (P > 1 && (size_t)P * spad_len(N) * csz > 96 * 1024) P /= 2;
    g.P_xy = P;
    int tz = (N / 2) / E;
    g.P_z = 256 / tz < 1 ? 1 : 256 / tz;
    // twiddles exp(-2 pi i m / N) from the host libm in double
    std::vector<double> tw(2 * N);
    for (int m = 0; m < N; m++) {
        double a = 2.0 * M_PI * (double)m / (double)N;
        tw[2 * m] = cos(a);
        tw[2 * m + 1] = -sin(a);
    }
    if (precision == MITOS_FP32) {
        std::vector<float> twf(2 * N);
        for (int i = 0; i < 2 * N; i++) twf[i] = (float)tw[i];
        if (cudaMalloc(&ge->tw, sizeof(float) * 2 * N) != cudaSuccess) { delete ge; set_error(5, "twiddles"); return nullptr; }
        cudaMemcpy(ge->tw, twf.data(), sizeof(float) * 2 * N, cudaMemcpyHostToDevice);
    } else {
        if (cudaMalloc(&ge->tw, sizeof(double) * 2 * N) != cudaSuccess) { delete ge; set_error(5, "twiddles"); return nullptr; }
        cudaMemcpy(ge->tw, tw.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice);
    }
    g.twN = ge->tw;
    ge->twst[0] = stage_twiddles(g.plN, tw, precision);
    ge->twst[1] = stage_twiddles(g.plH, tw, precision);
    {
        // the 16-element compile-time kernels' schedule (ct_radix_at), where it exists for N
        FFTPlan p16 = g.plN;
        p16.nst = 0;
        while (p16.nst < MITOS_MAX_STAGES && ct_radix_at(N, 16, p16.nst)) {
            p16.rad[p16.nst] = ct_radix_at(N, 16, p16.nst);
            p16.nst++;
        }
        int prod = 1;
        for (int s = 0; s < p16.nst; s++) prod *= p16.rad[s];
        ge->twst16 = prod == N ? stage_twiddles(p16, tw, precision) : nullptr;
    }
    if (!ge->twst[0] || !ge->twst[1]) {
        cudaGetLastError();
        delete ge;
        set_error(5, "stage twiddles");
        return nullptr;
    }
    g.plN.twst = ge->twst[0];
    g.plH.twst = ge->twst[1];
    g.plN.twst16 = ge->twst16;
    g.plH.twst16 = nullptr;
    g_geoms[key] = ge;
    return &ge->g;
}

int set_tiles(int N, int precision, int p_xy, int p_z) {
    const GridGeom *gc = geom(N, precision);
    if (!gc) return 3;
    const int tpp = N / gc->E, tz = (N / 2) / gc->E;
    const size_t csz = precision == MITOS_FP32 ? 8 : 16;
    // X / Y kernels: at most 512 threads and 96 KB of exchange buffer; Z kernels: 256 threads; all
    // blocks whole warps (the per-warp P(k) histograms and the warp-shuffle reductions need them)
    if (p_xy < 1 || p_xy * tpp > 512 || (p_xy * tpp) % 32 || (size_t)p_xy * spad_len(N) * csz > 96 * 1024 ||
        p_z < 1 || p_z * tz > 256 || (p_z * tz) % 32 || (size_t)p_z * spad_len(N / 2) * csz > 96 * 1024) {
        set_error(1, "tile %d x %d does not fit N = %d", p_xy, p_z, N);
        return 1;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    GridGeom *g = const_cast<GridGeom *>(gc);
    g->P_xy = p_xy;
    g->P_z = p_z;
    return 0;
}

int set_radix(int N, int precision, const int *rad_n, int ns_n, const int *rad_h, int ns_h) {
    const GridGeom *gc = geom(N, precision);
    if (!gc) return 3;
    FFTPlan pn, ph;
    if (!rad_n || !rad_h || !plan_from_radices(N, gc->E, N, rad_n, ns_n, &pn) ||
        !plan_from_radices(N / 2, gc->E, N, rad_h, ns_h, &ph)) {
        set_error(1, "radix schedule does not fit N = %d (radices 2, 3, 4, 8 dividing %d, product N and N/2)", N,
                  gc->E);
        return 1;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    GridGeom *g = const_cast<GridGeom *>(gc);
    FFTPlan dn, dh;
    make_plan(N, g->E, N, &dn);
    make_plan(N / 2, g->E, N, &dh);
    auto same = [](const FFTPlan &a, const FFTPlan &b) {
        if (a.nst != b.nst) return false;
        for (int i = 0; i < a.nst; i++)
            if (a.rad[i] != b.rad[i]) return false;
        return true;
    };
    // the stage tables belong to the default schedules, the only ones the compile-time kernels run
    pn.twst = g->plN.twst;
    ph.twst = g->plH.twst;
    pn.twst16 = g->plN.twst16;
    ph.twst16 = g->plH.twst16;
    g->plN = pn;
    g->plH = ph;
    g->custom_radix = !(same(pn, dn) && same(ph, dh));
    return 0;
}

int get_radix(int N, int precision, int *rad_n, int *ns_n, int *rad_h, int *ns_h) {
    const GridGeom *g = geom(N, precision);
    if (!g) return 3;
    *ns_n = g->plN.nst;
    *ns_h = g->plH.nst;
    for (int i = 0; i < MITOS_MAX_STAGES; i++) {
        rad_n[i] = i < g->plN.nst ? g->plN.rad[i] : 0;
        rad_h[i] = i < g->plH.nst ? g->plH.rad[i] : 0;
    }
    return 0;
}

int get_tiles(int N, int precision, int *p_xy, int *p_z) {
    const GridGeom *g = geom(N, precision);
    if (!g) return 3;
    *p_xy = g->P_xy;
    *p_z = g->P_z;
    return 0;
}

// 1 / sinc(pi m / N)^order, m = -N/2 .. N/2, stored at m + N/2
// (include/fft_kernels.h:187,198-219 factorised per axis)
static std::map<std::tuple<int, int, int>, void *> g_windows;
const void *window_table(int N, int order, int precision) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_tuple(N, order, precision);
    auto it = g_windows.find(key);
    if (it != g_windows.end()) return it->second;
    std::vector<double> w(N + 1);
    for (int m = -N / 2; m <= N / 2; m++) {
        double x = M_PI * (double)m / (double)N;
        double s = (m == 0) ? 1.0 : sin(x) / x;
        w[m + N / 2] = 1.0 / pow(s, order);
    }
    void *d = nullptr;
    if (precision == MITOS_FP32) {
        std::vector<float> wf(w.begin(), w.end());
        if (cudaMalloc(&d, sizeof(float) * (N + 1)) != cudaSuccess) return nullptr;
        cudaMemcpy(d, wf.data(), sizeof(float) * (N + 1), cudaMemcpyHostToDevice);
    } else {
        if (cudaMalloc(&d, sizeof(double) * (N + 1)) != cudaSuccess) return nullptr;
        cudaMemcpy(d, w.data(), sizeof(double) * (N + 1), cudaMemcpyHostToDevice);
    }
    g_windows[key] = d;
    return d;
}

// Fourier transfer of the on-node TSC stencil (1/8, 3/4, 1/8): 3/4 + cos(2 pi m / N) / 4,
// m = -N/2 .. N/2 stored at m + N/2
static std::map<std::pair<int, int>, void *> g_stencils;
const void *stencil_table(int N, int precision) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_pair(N, precision);
    auto it = g_stencils.find(key);
    if (it != g_stencils.end()) return it->second;
    std::vector<double> w(N + 1);
    for (int m = -N / 2; m <= N / 2; m++) w[m + N / 2] = 0.75 + 0.25 * cos(2.0 * M_PI * (double)m / (double)N);
    void *d = nullptr;
    if (precision == MITOS_FP32) {
        std::vector<float> wf(w.begin(), w.end());
        if (cudaMalloc(&d, sizeof(float) * (N + 1)) != cudaSuccess) return nullptr;
        cudaMemcpy(d, wf.data(), sizeof(float) * (N + 1), cudaMemcpyHostToDevice);
    } else {
        if (cudaMalloc(&d, sizeof(double) * (N + 1)) != cudaSuccess) return nullptr;
        cudaMemcpy(d, w.data(), sizeof(double) * (N + 1), cudaMemcpyHostToDevice);
    }
    g_stencils[key] = d;
    return d;
}

// bin of each squared integer wavevector norm n2 in [0, 3 (N/2)^2]; -1 skips the mode
static long isqrt_l(long a) {
    long r = (long)sqrt((double)a);
    while (r * r > a) r--;
    while ((r + 1) * (r + 1) <= a) r++;
    return r;
}
int pk_bin_of_n2(long n2, int N, int bins, int linear, double dk, double lmin, double lmax) {
    int b;
    if (linear) {
        // linear shells of width k_Nyquist / bins: b = isqrt(n2 bins^2) / (N/2)
        b = (int)(isqrt_l(n2 * (long)bins * bins) / (N / 2));
    } else {
        // src/calc_powerspec.c:61-63 with k = dk sqrt(n2)
        const double k = sqrt((double)n2) * dk;
        const float u = (log(k) - lmin) / (lmax - lmin);
        b = (int)floor((bins - 1) * u);
    }
    return (b >= 0 && b < bins) ? b : -1;
}

struct BinEntry {
    int *dev = nullptr;
    std::vector<int> host;
    std::vector<double> ksum;        // sum over modes of multiplicity * |k| per bin
    std::vector<long long> count;    // sum over modes of multiplicity per bin
    std::vector<long> lo, hi;        // |n|^2 range of each bin (lo > hi: empty)
    std::vector<char> contiguous;    // the bin's |n|^2 values form that one range
};
static std::map<std::tuple<int, int, int, double>, BinEntry *> g_bins;
static std::map<int, std::vector<long long>> g_n2hist;

static BinEntry *bin_entry(int N, int bins, int linear, double boxlen) {
    auto key = std::make_tuple(N, bins, linear, boxlen);
    auto it = g_bins.find(key);
    if (it != g_bins.end()) return it->second;
    const long n2max = 3L * (N / 2) * (N / 2);
    BinEntry *be = new BinEntry;
    std::vector<int> &tab = be->host;
    tab.assign(n2max + 1, -1);
    const double dk = 2 * M_PI / boxlen;
    const double max_k = sqrt(3) * dk * N / 2, min_k = dk;
    const double lmax = log(max_k), lmin = log(min_k);
    for (long n2 = 1; n2 <= n2max; n2++) tab[n2] = pk_bin_of_n2(n2, N, bins, linear, dk, lmin, lmax);
    if (cudaMalloc(&be->dev, sizeof(int) * (n2max + 1)) != cudaSuccess) {
        cudaGetLastError();
        delete be;
        return nullptr;
    }
    cudaMemcpy(be->dev, tab.data(), sizeof(int) * (n2max + 1), cudaMemcpyHostToDevice);
    // multiplicity-weighted mode count per n2 over the half-complex grid (weight 2 except on the
    // kz = 0 and kz = N/2 planes, src/calc_powerspec.c:73-79), then per bin
    auto &hist = g_n2hist[N];
    if (hist.empty()) {
        hist.assign(n2max + 1, 0);
        for (int x = 0; x < N; x++) {
            const long jx = x > N / 2 ? x - N : x;
            for (int y = 0; y < N; y++) {
                const long jy = y > N / 2 ? y - N : y;
                const long b2 = jx * jx + jy * jy;
                for (int z = 0; z <= N / 2; z++) hist[b2 + (long)z * z] += (z == 0 || z == N / 2) ? 1 : 2;
            }
        }
    }
    be->lo.assign(bins, 1);
    be->hi.assign(bins, 0);
    be->contiguous.assign(bins, 1);
    for (long n2 = 1; n2 <= n2max; n2++) {
        const int b = tab[n2];
        if (b < 0) continue;
        if (be->lo[b] > be->hi[b]) be->lo[b] = n2;
        else if (be->hi[b] != n2 - 1) be->contiguous[b] = 0;
        be->hi[b] = n2;
    }
    be->ksum.assign(bins, 0.0);
    be->count.assign(bins, 0);
    for (long n2 = 1; n2 <= n2max; n2++) {
        const int b = tab[n2];
        if (b < 0 || !hist[n2]) continue;
        be->count[b] += hist[n2];
        be->ksum[b] += (double)hist[n2] * sqrt((double)n2) * dk;
    }
    g_bins[key] = be;
    return be;
}

const int *bin_table(int N, int bins, int linear, double boxlen) {
    std::lock_guard<std::mutex> lk(g_mu);
    BinEntry *be = bin_entry(N, bins, linear, boxlen);
    return be ? be->dev : nullptr;
}

int bin_n2_range(int N, int bins, int linear, double boxlen, int b, long *lo, long *hi) {
    std::lock_guard<std::mutex> lk(g_mu);
    BinEntry *be = bin_entry(N, bins, linear, boxlen);
    if (!be) return 5;
    if (b < 0 || b >= bins) {  // no mode falls in a bin outside the table: an empty range
        *lo = 1;
        *hi = 0;
        return 0;
    }
    if (!be->contiguous[b]) {
        set_error(3, "bin %d is not one range of |n|^2", b);
        return 3;
    }
    *lo = be->lo[b];
    *hi = be->hi[b];
    return 0;
}

int bin_geometry(int N, int bins, int linear, double boxlen, const double **ksum, const long long **count) {
    std::lock_guard<std::mutex> lk(g_mu);
    BinEntry *be = bin_entry(N, bins, linear, boxlen);
    if (!be) return 5;
    *ksum = be->ksum.data();
    *count = be->count.data();
    return 0;
}

// ---- the Z passes' row-copy fault word ---------------------------------------------------
static int *g_zrow_fault_host = nullptr, *g_zrow_fault_dev = nullptr;
int *zrow_fault_device() {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_zrow_fault_host) {
        int *hp = nullptr, *dp = nullptr;
        if (cudaHostAlloc((void **)&hp, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (cudaHostGetDevicePointer((void **)&dp, hp, 0) != cudaSuccess) {
            cudaGetLastError();
            cudaFreeHost(hp);
            return nullptr;
        }
        *hp = 0;
        g_zrow_fault_host = hp;
        g_zrow_fault_dev = dp;
    }
    return g_zrow_fault_dev;
}
int zrow_fault_check() {
    if (!g_zrow_fault_host || !*(volatile int *)g_zrow_fault_host) return 0;
    *g_zrow_fault_host = 0;
    set_error(6, "a Z pass's row copy did not complete (bounded wait timed out; rows read from global memory)");
    return 6;
}

// ---- workspace: grid-sized device buffers reused across calls --------------------------
static std::map<std::pair<size_t, int>, std::vector<void *>> g_ws;
void *workspace(size_t bytes, int slot) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto &v = g_ws[std::make_pair(bytes, t_ws_set)];
    while ((int)v.size() <= slot) v.push_back(nullptr);
    if (!v[slot]) {
        if (cudaMalloc(&v[slot], bytes) != cudaSuccess) {
            cudaGetLastError();
            v[slot] = nullptr;
            set_error(5, "out of device memory allocating a %zu-byte workspace", bytes);
        }
    }
    return v[slot];
}

void release_all() {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto &kv : g_ws)
        for (void *p : kv.second) if (p) cudaFree(p);
    g_ws.clear();
    for (auto &kv : g_geoms) { cudaFree(kv.second->tw); delete kv.second; }
    g_geoms.clear();
    for (auto &kv : g_windows) cudaFree(kv.second);
    g_windows.clear();
    for (auto &kv : g_stencils) cudaFree(kv.second);
    g_stencils.clear();
    for (auto &kv : g_bins) { cudaFree(kv.second->dev); delete kv.second; }
    g_bins.clear();
}

}  // namespace mitos

extern "C" const char *mitos_last_error(void) { return mitos::g_err; }

// per-launch timing (off by default): enable, run, then read name / milliseconds pairs
extern "C" int mitos_kernel_timing(int on) {
    cudaStreamSynchronize(mitos::stream());
    for (auto &k : mitos::g_kev) {
        cudaEventDestroy(k.second.first);
        cudaEventDestroy(k.second.second);
    }
    mitos::g_kev.clear();
    mitos::g_ktime = on != 0;
    return 0;
}
extern "C" int mitos_kernel_times(const char **names, double *ms, int max) {
    cudaStreamSynchronize(mitos::stream());
    int n = 0;
    for (auto &k : mitos::g_kev) {
        if (n >= max) break;
        float m = 0;
        cudaEventElapsedTime(&m, k.second.first, k.second.second);
        names[n] = k.first;
        ms[n] = m;
        n++;
    }
    return n;
}
extern "C" long mitos_launch_count(void) { return mitos::g_launches; }
extern "C" int mitos_release_all(void) {
    cudaDeviceSynchronize();
    mitos::release_all();
    mitos::release_jump_tables();
    mitos::release_thermal_tables();
    return 0;
}

// CUDA-event timer on the library stream (the stream every kernel of the library runs on)
static cudaEvent_t g_t0 = nullptr, g_t1 = nullptr;
extern "C" int mitos_timer_start(void) {
    if (!g_t0) {
        cudaEventCreate(&g_t0);
        cudaEventCreate(&g_t1);
    }
    return cudaEventRecord(g_t0, mitos::stream()) == cudaSuccess ? 0 : 4;
}
extern "C" double mitos_timer_stop(void) {
    cudaEventRecord(g_t1, mitos::stream());
    cudaEventSynchronize(g_t1);
    float ms = 0;
    cudaEventElapsedTime(&ms, g_t0, g_t1);
    return ms;
}
extern "C" int mitos_sync(void) {
    return cudaStreamSynchronize(mitos::stream()) == cudaSuccess ? 0 : 4;
}
