// grid2d.h - host-visible part of the grid-wide persistent kernel of small
// 2D grids (grid2d.cuh): the launch arguments and the launchers.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace gpe {

constexpr int G2_THREADS = 256;

// One realisation (context) of the batch.  Both passes run on the default
// plans Plan<n>; the context's tables are built for them.
struct G2Grid {
  void* psi;                 // cx<R> state, ny x nx, y fastest
  const void* V;             // R potential
  const void* tws[2];        // stage twiddle rows: [0] x axis, [1] y axis
  const void* php[2];        // kinetic factors exp(-k^2/2 dt)/n in slot order
  const void* k2p[2];        // k^2/2/n in slot order (energy sums)
  DevScalars* sc;
  double* partials;          // [NSLOTS + 1][cap] per-tile partial sums of this context
  double* hist;              // record (muc, ncur, energy) of outer step k at hist + 3*k
  int cap;
  int nx, ny;
  int ytiles, xtiles;        // tiles of the y pass (x columns) and of the x pass (y rows)
  int feedback;              // gamma > 0 and mu_init == 0: mu and the norm feed back every block
  int start;                 // current_iter at the start of the run
  double weight, g, tau;     // cell volume, coupling, decay time (0: none)
  double dre, dim;           // complex time step dt = i ddt/(1 + i gamma)
};

struct G2Args {
  const G2Grid* grids;
  int ngrids;
  const int* yoff;  // [ngrids + 1] first y item of each grid (prefix sums of ytiles)
  const int* xoff;  // [ngrids + 1] first x item of each grid
  int n_rec, nb;    // steps per block, blocks per outer step
  int nouter;       // outer steps per launch
  double ddt, dt_outer;
  unsigned* bar;    // [0] grid-barrier arrival counter, [1] work-item counter; zero at launch
  int* fail;        // set when a grid barrier's bounded wait ran out
  int epi_y = 0;    // the block-end epilogue ran on the y pass (folded steps, even n_rec)
};

// Pencils per tile of the y pass (contiguous) and the x pass (strided) for
// an axis length of the persistent kernel (0: length not handled).
int grid2d_tile_pencils(int n, bool strided);
// Dynamic shared memory of the kernel (the largest pass body).
size_t grid2d_smem();
// CTAs of a cooperative launch that fit the device at once.
int grid2d_max_ctas();
// Cooperative launch of nctas CTAs.
cudaError_t launch_grid2d(const G2Args& a, int nctas, cudaStream_t s);
// The launches of one block of n_rec steps on the multi-grid pass kernels,
// for a group of grids of one shape (ny x nx): per step a y pass and an x
// pass over the group's tiles, then (energy: some grid of the group needs mu
// at this block end) the kinetic sums, and the block finalizer of every grid
// (jj: the block's index in the outer step, last: the outer step's last
// block).
// fold: folded steps (y x, x y, ...; the shared axis of consecutive steps
// as one pass).
cudaError_t launch_multi2d_block(const G2Args& a, int ny, int nx, int ny_items, int nx_items, int jj, bool last,
                                 bool energy, bool fold, cudaStream_t s);

}  // namespace gpe
