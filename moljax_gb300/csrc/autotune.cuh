// Process-wide registry of autotuned launch choices (host only).
//
// The autotuner times candidate configurations of a kernel on the device with CUDA
// events and installs the fastest here; the launchers read it when they build their
// arguments, so a tuned choice applies to every later call for that size.  Entries:
//   * mixed-radix DFTs (dftn.cu): the radix schedule of length n (order of the radix
//     2/3/4/5 passes and whether powers of two go as 4s or 2s) and the threads per
//     sequence;
//   * stencil stages (explicit.cu): the rows per warp strip of rk_stage_kernel, i.e.
//     the tile height, per grid size, field count and element size.
#pragma once

namespace mjx {

struct DftTune {
  int nrad;     // 0: no schedule installed
  int rad[16];
  int tpsm;     // threads per sequence (0: default n/8)
};

bool tune_dft_get(int n, int elem, DftTune* t);
void tune_dft_put(int n, int elem, const DftTune& t);
void tune_dft_clear(int n, int elem);
int tune_rows_get(int ny, int nx, int nf, int elem);  // 0 when untuned
void tune_rows_put(int ny, int nx, int nf, int elem, int rows);
// candidate radix schedules of n: rows of 17 ints [nrad, r0 .. r15]; returns the count
int dft_schedules(int n, int* out, int max);

}  // namespace mjx
