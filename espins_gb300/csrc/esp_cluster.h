// Cluster-resident sweep kernel (esp_cluster.cu): arguments and launchers.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "esp_device.cuh"

namespace esp {

constexpr int kClusterThreads = 512;
constexpr int kMaxClusterAtoms = 8;
constexpr int kMaxStencil = 64;
constexpr int kMaxClasses = 8 * kMaxClusterAtoms;

// Couplings of stencil entry e of parity class k (the neighbour's position
// comes from the index table); padded to 32 bytes.
struct ClusterNbr {
    float J, B, Dx, Dy, Dz, pad0, pad1, pad2;
};

// Everything the kernel needs about the lattice's couplings; the header is
// followed in memory by nclass * maxst ClusterNbr entries (class-major).
struct ClusterStencil {
    int nclass, maxst, ncolour, pad;
    int count[kMaxClasses];            // entries of each class
    float4 si[kMaxClusterAtoms];       // (ax, ay, az, Delta)
    float4 fld[kMaxClusterAtoms];      // (f ax, f ay, f az, 0)
    float mag[kMaxClusterAtoms];
    int colour_start[kMaxClasses + 1]; // classes of colour c: class_order[colour_start[c] .. colour_start[c+1])
    int class_order[kMaxClasses];
};

// The z planes of a replica over the cs CTAs of its cluster: ranks
// [0, nA) hold pz planes, the others pz - 2 (pz even; nA == cs when every
// slab is equal), so any even Lz with Lz / 2 >= cs splits.  Local sites of a
// rank follow those of the ranks before it in the replica's slab order.
__host__ __device__ inline int slab_planes(int pz, int nA, int q) { return q < nA ? pz : pz - 2; }
__host__ __device__ inline int slab_z0(int pz, int nA, int q) { return q < nA ? q * pz : nA * pz + (q - nA) * (pz - 2); }

inline size_t cluster_stencil_bytes(int nclass, int maxst)
{
    return sizeof(ClusterStencil) + (size_t)nclass * maxst * sizeof(ClusterNbr);
}

struct ClusterArgs {
    const ClusterStencil *stencil;  // device copy (header + entries)
    int stencil_words;              // size of that copy in 4-byte words
    // [rank][entry / 4][local site][entry % 4]: the neighbour's local index,
    // | 0x80000000 | (owner rank << 24) when the owner is a peer CTA
    const uint32_t *nbidx;
    int Lx, Ly, Lz, na, N, R, nclass, pz, nA;  // slab_planes(pz, nA, rank) z planes per CTA
    int has_b, has_d, has_si, has_f;
    // state: the slabs of every replica, [r][rank][local site][x, y, z],
    // converted from and to the handle's spin arrays around the launch; or,
    // with slab == null (small slabs, where two more launches cost more than
    // they save), the spin arrays themselves, element (p, r) at p*R + r
    float *slab;
    float *sx, *sy, *sz;
    const int32_t *inv;             // reference site -> p
    const int32_t *temp_of;
    const float *beta;
    double *e_run, *m_run;
    unsigned long long *rej;        // [R slots][2]
    int phase;
    // measurement
    int measure, n_meas, steps_measure;
    long long meas_base;
    double *data, *lsum, *binning;
    const int32_t *levels;
    int nlev, pt_quirk;
    unsigned long long *pm_counts;
    double *series;                 // [cap][R slots][2] or null
    long long series_cap;
    int nf;
    double m_min, m_max;
    // random stream
    unsigned long long sweep_base;
    // device counters [sweep, swap, measurement, unit] added to sweep_base
    // and meas_base, or null
    const unsigned long long *ctr;
    // divisions by per-class sites (ranks < nA, the others) and half-cell extents
    FastDiv fd_pc, fd_pc2, fd_hx, fd_hy;
    double rn_inv;                  // 1 / N
    uint32_t key0, key1;
    int mode;
    float tilt;
    // optional measurements (mcarlo.F90:553-578): bit 0 order parameter,
    // bit 1 staggered magnetisation
    int obs;
    const float4 *obs_atom;         // [na]: axis (x, y, z), staggered coefficient (w)
    double *obs_data;               // [R slots][6]
    double *obs_lsum, *obs_bin;     // [R slots][nlev][2]
    unsigned long long *obs_pm;     // [R slots][2][nf]
};

// The handle's spin arrays (element (p, r) at p*R + r, p = inv[reference
// site]) to and from the slab layout of the cluster path, [r][rank][l][3]
// with l the kernel's local site order (class-major, then half-cell x, y, z
// within the rank's planes): shared-memory transposes of 32 sites x 32
// replicas, coalesced on both sides.
struct SlabArgs {
    float *sx, *sy, *sz;
    float *slab;
    const int32_t *inv;
    int Lx, Ly, na, R, pz, nA, cs, N, n_local;   // n_local: the largest rank's sites
    FastDiv fd_pc, fd_pc2, fd_hx, fd_hy;
};
cudaError_t launch_to_slabs(const SlabArgs &a, cudaStream_t st);
cudaError_t launch_from_slabs(const SlabArgs &a, cudaStream_t st);

// nhist: P(M) histogram only (1) or P(M), P(OP), P(SM) (3)
// binning levels whose sums a cluster keeps in shared memory during a launch
// (more levels are updated in global memory)
constexpr int kClusterMaxLev = 32;
// doubles of that cache: data and obs data (12), levels (16), four [level][2] arrays
constexpr int kClusterAccDoubles = 12 + kClusterMaxLev / 2 + 8 * kClusterMaxLev;
// doubles of the reduction scratch before that cache
constexpr int kClusterRedDoubles = 152;
size_t cluster_smem_bytes(int n_local, int nf, int nhist, size_t stencil_bytes);
// nt: threads per CTA, 256 or 512
// The dynamic shared-memory limit is a property of a kernel function, shared
// by every handle that launches it: raise it to the most the device allows
// next to the kernel's static shared memory (it is an upper bound, not an
// allocation), so that configuring one handle never lowers the limit another
// handle's launches need.  Fails if `need` exceeds that maximum.
inline cudaError_t allow_max_dynamic_smem(const void *kernel, size_t need)
{
    int dev = 0, v = 0;
    cudaFuncAttributes fa{};
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    const long long room = (long long)v - (long long)fa.sharedSizeBytes;
    if (room <= 0 || need > (size_t)room) return cudaErrorInvalidValue;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room);
}

// Thread geometries of the kernel: nt threads per CTA, S sites of a colour
// pass per thread (updated together): (256, 1), (512, 1), (512, 2).
bool cluster_threads_ok(int nt, int S);
cudaError_t cluster_configure(size_t smem, int csize, int nt, int S);
// Clusters of csize CTAs of nt threads with `smem` bytes each that fit on the GPU at once.
int cluster_max_active(int csize, int nt, int S, size_t smem, int R);
cudaError_t launch_cluster(const ClusterArgs &a, int csize, int nt, int S, size_t smem, cudaStream_t st);

}  // namespace esp
