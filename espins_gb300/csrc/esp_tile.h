// Tiled sweep kernel (esp_tile.cu): arguments and launchers.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "esp_cluster.h"
#include "esp_device.cuh"

namespace esp {

struct TileArgs {
    const ClusterStencil *stencil;  // device copy of the cluster path's stencil (header + entries)
    // per atom: entries with biquadratic or DM couplings first (nbd8 of them,
    // padded to a multiple of 8), then exchange-only entries up to nall8;
    // padding entries are the site itself with zero couplings.  nbd2: the
    // first part's entries rounded up to 2; nall4: nbd8 + the second part's
    // rounded up to 4 (the kernels that step 2 and 4 entries at a time skip
    // the rest of the padding)
    const int4 *offs;               // [na][maxst]: (dx, dy, dz, target atom) in cells
    const ClusterNbr *cpl;          // [na][maxst] couplings in the same order
    int maxst;
    int nbd8[kMaxClusterAtoms], nall8[kMaxClusterAtoms];
    int nbd2[kMaxClusterAtoms], nall4[kMaxClusterAtoms];
    int Lx, Ly, Lz, na, N, R;
    int T, G;                       // tile edge (cells, even), replicas per CTA
    int ntx, nty, ntz;              // tiles per axis (even)
    int phase;                      // tile parity: bit 0 x, bit 1 y, bit 2 z
    int has_b, has_d, has_si, has_f;
    float *sx, *sy, *sz;
    const int32_t *inv;             // reference site -> p
    const int32_t *temp_of;
    const float *beta;
    double *part;                   // [tiles][R][4]: dE, dMx, dMy, dMz
    unsigned long long *part_rej;   // [tiles][R]
    unsigned long long sweep;
    const unsigned long long *ctr;  // device sweep counter added to sweep, or null
    uint32_t key0, key1;
    int mode;
    float tilt;
};

// The tiles' slots are folded in two passes: chunks of kTileFoldChunk tiles
// (one block each, consecutive threads on consecutive slot words), then the
// chunks in order; part and part_rej hold tile_fold_chunks(ntiles) chunk
// slots after the tiles' own.
constexpr int kTileFoldChunk = 32;
__host__ __device__ inline int tile_fold_chunks(int ntiles) { return (ntiles + kTileFoldChunk - 1) / kTileFoldChunk; }

struct TileFoldArgs {
    double *part;                   // [ntiles + chunks][R][4]
    unsigned long long *part_rej;   // [ntiles + chunks][R]
    double *e_run, *m_run;
    unsigned long long *rej;
    const int32_t *temp_of;
    int R, ntiles, phase;
};

size_t tile_smem_bytes(int T, int G, int na, int maxst);
cudaError_t tile_configure(size_t smem);
// one launch = the tiles of one parity (a.phase); eight make a sweep
cudaError_t launch_tile(const TileArgs &a, size_t smem, cudaStream_t st);
cudaError_t launch_tile_fold(const TileFoldArgs &a, cudaStream_t st);
// pipelined persistent variant (T in {4, 6, 8}, G in {4, 8, 16}); nb box
// buffers per CTA: 2 = one CTA per SM with the next box copied during the
// updates, 1 = two CTAs per SM
size_t tile_p_smem_bytes(int T, int G, int na, int maxst, int nb);
bool tile_p_supported(int T, int G, int na);
cudaError_t tile_p_configure(int T, int G, int nb, size_t smem);
// the persistent grid of a geometry (a's shape, T, G, R and term flags):
// as many CTAs as the GPU holds at once, at most one per item
cudaError_t tile_p_grid(const TileArgs &a, size_t smem, int num_sms, int nb, int *blocks);
cudaError_t launch_tile_p(const TileArgs &a, size_t smem, int blocks, int nb, cudaStream_t st);

}  // namespace esp
