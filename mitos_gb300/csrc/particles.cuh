// particles.cuh -- particle stage launchers.
#pragma once

namespace mitos {

// lattice of M^3 particles, TSC displacement by the three padded displacement grids, wrap,
// CIC into rho (padded real grid, accumulated, in units of the mean density); pos_out optional
int displace_and_deposit(int N, int M, double boxlen, int precision, const void *d0, const void *d1,
                         const void *d2, void *rho, float *pos_out, float *posraw_out = nullptr);
// lattice-aligned fast path (M = N, exact nodes); the displacement grids must carry the folded
// on-node TSC stencils (PassArgs::stencil in the displacement passes)
// disp_pitch / rho_pitch: row pitches (elements) of the displacement grids and of rho, 16-byte multiples
// batch > 1: that many realisations, every grid (d0, d1, d2, rho) bstride bytes apart; pos_out null
// posraw_out (optional): the positions before the wrap (the velocity gather's), M^3 x 3
int lattice_deposit(int N, double boxlen, int precision, const void *d0, const void *d1, const void *d2,
                    int disp_pitch, void *rho, int rho_pitch, float *pos_out, int batch = 1, size_t bstride = 0,
                    float *posraw_out = nullptr);
bool lattice_aligned(int N, int M, double boxlen);
// tensor-copy staging of the deposit's interior bricks on (default) or off (16-byte cp.async)
void set_lattice_tma(bool on);
bool lattice_tma();
// brick order of the deposit: 8 x 8 x 4 regions (default) or x, y, z rows (identical output in FP32)
void set_lattice_region(bool on);
bool lattice_region();
// a deposit that stops because a tile copy never completed (bounded wait) sets a device flag:
// lattice_fault_fetch queues its copy to the host behind the deposit; lattice_fault_check, once the
// library stream is synchronised, returns 6 with the error message if it was set (and clears it)
int lattice_fault_fetch();
int lattice_fault_check();
// particle velocities: TSC gather of the three velocity grids (row pitch `pitch` reals) at the
// unwrapped positions pos (np x 3), float velocities out (np x 3)
int velocity_gather(long np, int N, int pitch, double boxlen, int precision, const float *pos, const void *v0,
                    const void *v1, const void *v2, float *vel);
// CIC of n given positions with per-particle value val
int cic_positions(long n, int N, double boxlen, int precision, const float *pos, double val, void *rho);
// snapshot particle datasets (src/mitos.c:1106-1117) from device positions / velocities (vel may be
// null: zero velocities); outputs device, any may be null
int snapshot_arrays(long n, const float *pos, const float *vel, float mass, long long id_first, double *coords,
                    double *vels, double *masses, long long *ids);
// n floats to doubles (device)
int widen_to_double(long n, const float *src, double *dst);

}  // namespace mitos
