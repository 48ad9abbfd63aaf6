/*
 * manet_oracle.c -- FP64 restatement of the Monge-Ampere warm-start network (see manet_oracle.h).
 * TEST INFRASTRUCTURE ONLY.
 */
#include "manet_oracle.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

static const int CIN[4] = {3, 16, 16, 16};
static const int COUT[4] = {16, 16, 16, 1};

double orc_bf16(double x) {
    float f = (float)x;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x; /* inf / nan unchanged */
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    memcpy(&f, &u, 4);
    return (double)f;
}

static inline long wrap(long i, long N) { return i < 0 ? i + N : (i >= N ? i - N : i); }

/* voxel index of v shifted by tap t */
static inline long shift(int N, long x, long y, long z, int t, int sign) {
    const long dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
    return (wrap(x + sign * dx, N) * N + wrap(y + sign * dy, N)) * N + wrap(z + sign * dz, N);
}

void orc_conv3d(int N, int cin, int cout, const double *in, const double *w, const double *b, int relu,
                double *out) {
    const long nv = (long)N * N * N;
#pragma omp parallel for schedule(static)
    for (long v = 0; v < nv; v++) {
        const long x = v / ((long)N * N), y = (v / N) % N, z = v % N;
        double acc[64];
        for (int co = 0; co < cout; co++) acc[co] = b ? b[co] : 0.0;
        for (int t = 0; t < 27; t++) {
            const double *src = in + shift(N, x, y, z, t, +1) * cin;
            for (int ci = 0; ci < cin; ci++) {
                const double a = src[ci];
                const double *wr = w + ((long)t * cin + ci) * cout;
                for (int co = 0; co < cout; co++) acc[co] += a * wr[co];
            }
        }
        for (int co = 0; co < cout; co++) out[v * cout + co] = (relu && acc[co] < 0) ? 0.0 : acc[co];
    }
}

void orc_conv3d_bwd_data(int N, int cin, int cout, const double *dout, const double *w, double *din) {
    const long nv = (long)N * N * N;
#pragma omp parallel for schedule(static)
    for (long v = 0; v < nv; v++) {
        const long x = v / ((long)N * N), y = (v / N) % N, z = v % N;
        double acc[64];
        for (int ci = 0; ci < cin; ci++) acc[ci] = 0.0;
        for (int t = 0; t < 27; t++) {
            const double *g = dout + shift(N, x, y, z, t, -1) * cout;
            for (int ci = 0; ci < cin; ci++) {
                const double *wr = w + ((long)t * cin + ci) * cout;
                double s = 0;
                for (int co = 0; co < cout; co++) s += g[co] * wr[co];
                acc[ci] += s;
            }
        }
        for (int ci = 0; ci < cin; ci++) din[v * cin + ci] = acc[ci];
    }
}

void orc_conv3d_bwd_weight(int N, int cin, int cout, const double *in, const double *dout, double *dw,
                           double *db) {
    const long nv = (long)N * N * N;
    const int nw = 27 * cin * cout;
    memset(dw, 0, sizeof(double) * nw);
    if (db) memset(db, 0, sizeof(double) * cout);
    /* per-thread partial sums, added in thread order after the loop (deterministic) */
    const int nt = omp_get_max_threads();
    double *pw = calloc((size_t)nt * (nw + 64), sizeof(double));
#pragma omp parallel num_threads(nt)
    {
        double *mine = pw + (size_t)omp_get_thread_num() * (nw + 64);
#pragma omp for schedule(static)
        for (long v = 0; v < nv; v++) {
            const long x = v / ((long)N * N), y = (v / N) % N, z = v % N;
            const double *g = dout + v * cout;
            for (int co = 0; co < cout; co++) mine[nw + co] += g[co];
            for (int t = 0; t < 27; t++) {
                const double *src = in + shift(N, x, y, z, t, +1) * cin;
                for (int ci = 0; ci < cin; ci++) {
                    double *wr = mine + ((long)t * cin + ci) * cout;
                    for (int co = 0; co < cout; co++) wr[co] += src[ci] * g[co];
                }
            }
        }
    }
    for (int k = 0; k < nt; k++) {
        const double *p = pw + (size_t)k * (nw + 64);
        for (int i = 0; i < nw; i++) dw[i] += p[i];
        if (db)
            for (int co = 0; co < cout; co++) db[co] += p[nw + co];
    }
    free(pw);
}

double orc_manet_loss_grad(int N, const double *x, const double *target, const double *const *w,
                           const double *const *b, int round_bf16, double *pred, double *const *dw,
                           double *const *db) {
    const long nv = (long)N * N * N;
    double *wl[4];
    double *act[5]; /* act[0] = input, act[l+1] = output of layer l */
    for (int l = 0; l < 4; l++) {
        const int n = 27 * CIN[l] * COUT[l];
        wl[l] = malloc(sizeof(double) * n);
        for (int i = 0; i < n; i++) wl[l][i] = round_bf16 ? orc_bf16(w[l][i]) : w[l][i];
    }
    act[0] = malloc(sizeof(double) * nv * 3);
    for (long i = 0; i < nv * 3; i++) act[0][i] = round_bf16 ? orc_bf16(x[i]) : x[i];
    for (int l = 0; l < 4; l++) {
        act[l + 1] = malloc(sizeof(double) * nv * COUT[l]);
        orc_conv3d(N, CIN[l], COUT[l], act[l], wl[l], b[l], l < 3, act[l + 1]);
        if (round_bf16 && l < 3)
            for (long i = 0; i < nv * COUT[l]; i++) act[l + 1][i] = orc_bf16(act[l + 1][i]);
    }
    double loss = 0;
    double *g = malloc(sizeof(double) * nv);
    for (long v = 0; v < nv; v++) {
        const double d = act[4][v] - target[v];
        loss += d * d;
        g[v] = 2.0 * d / (double)nv;
        if (round_bf16) g[v] = orc_bf16(g[v]);
        if (pred) pred[v] = act[4][v];
    }
    loss /= (double)nv;
    /* backward: g holds dL/d(output of layer l) */
    for (int l = 3; l >= 0; l--) {
        orc_conv3d_bwd_weight(N, CIN[l], COUT[l], act[l], g, dw[l], db[l]);
        if (l == 0) break;
        double *gi = malloc(sizeof(double) * nv * CIN[l]);
        orc_conv3d_bwd_data(N, CIN[l], COUT[l], g, wl[l], gi);
        /* ReLU of the previous layer: gradient passes where its output is positive */
        for (long i = 0; i < nv * CIN[l]; i++) {
            gi[i] = act[l][i] > 0 ? gi[i] : 0.0;
            if (round_bf16) gi[i] = orc_bf16(gi[i]);
        }
        free(g);
        g = gi;
    }
    free(g);
    for (int l = 0; l < 5; l++) free(act[l]);
    for (int l = 0; l < 4; l++) free(wl[l]);
    return loss;
}
