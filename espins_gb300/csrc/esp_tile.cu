// Tiled sweeps for translation-invariant lattices too large for one cluster.
//
// The lattice is cut into cubes of T cells (T even, L a multiple of 2T along
// every axis).  A CTA stages one tile plus a one-cell halo of G replicas in
// shared memory, runs every colour class of the tile's sites against the
// frozen halo (each site once), and writes the tile back.  Tiles form a
// 2 x 2 x 2 checkerboard; one launch takes the tiles of one parity, so tiles
// updated at the same time are a tile apart and never interact, and a sweep is
// eight launches.  Every site is updated once per sweep with the Philox
// counter (site, replica, sweep) of the other sweep kernels and the same
// local-field arithmetic (delta_energy_get, get_quant.F90:294-333; metropolis,
// get_quant.F90:52-182); only the order of updates differs (tile by tile),
// which leaves the stationary distribution unchanged.
//
// HBM traffic per sweep: (T+2)^3 / T^3 reads + one write of every spin, so
// T = 8 costs ~35 B per site update against 24 B compulsory; the spins of the
// G replicas of a site are contiguous (element (p, r) at p*R + r).
#include "esp_tile.h"

#include <algorithm>

namespace esp {

namespace {

constexpr int kTileThreads = 256;

// One stencil entry's share of the local field g and of the quadratic form Q
// (delta_energy_get, get_quant.F90:294-297 exchange, :316-325 biquadratic,
// :327-333 DM) in one fixed sequence of IEEE operations, shared by the
// one-replica kernel (float) and the two-replica kernel (float2 lanes through
// fma.rn.f32x2), so the two give identical bits:
//   g   <- fma(-J, t, g)
//   Q_ab <- fma(B t_a, t_b, Q_ab)
//   g_x <- fma(t_z, -D_y, fma(t_y, D_z, g_x)), and cyclically for y, z
struct FieldQ {
    float gx, gy, gz, qxx, qyy, qzz, qxy, qxz, qyz;
};
struct FieldQ2 {
    float2 gx, gy, gz, qxx, qyy, qzz, qxy, qxz, qyz;
};

__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

__device__ __forceinline__ void entry_exchange(FieldQ &f, float nJ, float tx, float ty, float tz)
{
    f.gx = fmaf(nJ, tx, f.gx); f.gy = fmaf(nJ, ty, f.gy); f.gz = fmaf(nJ, tz, f.gz);
}
__device__ __forceinline__ void entry_bq(FieldQ &f, float Bv, float tx, float ty, float tz)
{
    bq_form(Bv, tx, ty, tz, f.qxx, f.qyy, f.qzz, f.qxy, f.qxz, f.qyz);
}
__device__ __forceinline__ void entry_dm(FieldQ &f, float dx, float dy, float dz, float tx, float ty, float tz)
{
    dm_field(dx, dy, dz, tx, ty, tz, f.gx, f.gy, f.gz);
}
__device__ __forceinline__ void entry_exchange(FieldQ2 &f, float2 nJ, float2 tx, float2 ty, float2 tz)
{
    f.gx = ffma2(nJ, tx, f.gx); f.gy = ffma2(nJ, ty, f.gy); f.gz = ffma2(nJ, tz, f.gz);
}
__device__ __forceinline__ void entry_bq(FieldQ2 &f, float2 Bv, float2 tx, float2 ty, float2 tz)
{
    const float2 bx = fmul2(Bv, tx), by = fmul2(Bv, ty), bz = fmul2(Bv, tz);
    f.qxx = ffma2(bx, tx, f.qxx); f.qyy = ffma2(by, ty, f.qyy); f.qzz = ffma2(bz, tz, f.qzz);
    f.qxy = ffma2(bx, ty, f.qxy); f.qxz = ffma2(bx, tz, f.qxz); f.qyz = ffma2(by, tz, f.qyz);
}
// nd = (-D_x, -D_y, -D_z) duplicated in both lanes
__device__ __forceinline__ void entry_dm(FieldQ2 &f, float2 dx, float2 dy, float2 dz, float2 ndx, float2 ndy,
                                         float2 ndz, float2 tx, float2 ty, float2 tz)
{
    f.gx = ffma2(tz, ndy, ffma2(ty, dz, f.gx));
    f.gy = ffma2(tx, ndz, ffma2(tz, dx, f.gy));
    f.gz = ffma2(ty, ndx, ffma2(tx, dy, f.gz));
}
__device__ __forceinline__ FieldQ lane_of(const FieldQ2 &f, int k)
{
    FieldQ o;
    o.gx = k ? f.gx.y : f.gx.x; o.gy = k ? f.gy.y : f.gy.x; o.gz = k ? f.gz.y : f.gz.x;
    o.qxx = k ? f.qxx.y : f.qxx.x; o.qyy = k ? f.qyy.y : f.qyy.x; o.qzz = k ? f.qzz.y : f.qzz.x;
    o.qxy = k ? f.qxy.y : f.qxy.x; o.qxz = k ? f.qxz.y : f.qxz.x; o.qyz = k ? f.qyz.y : f.qyz.x;
    return o;
}

// The Metropolis trial of one site of replica r (metropolis, get_quant.F90:52-182)
// given its exchange/biquadratic/DM field: adds the single-ion and field
// terms, draws the trial spin, and returns whether it is accepted, with the new
// spin n and the energy change de.
__device__ __forceinline__ bool tile_trial(const TileArgs &a, const ClusterStencil *st, FieldQ f, int at,
                                           uint32_t orig, uint32_t r, uint32_t sw_lo, uint32_t sw_hi, float beta,
                                           float ox, float oy, float oz, float &nx, float &ny, float &nz, float &de,
                                           bool hb)
{
    if (a.has_si) si_form(st->si[at], f.qxx, f.qyy, f.qzz, f.qxy, f.qxz, f.qyz);
    if (a.has_f) {
        const float4 fl = st->fld[at];
        f.gx = __fadd_rn(f.gx, fl.x); f.gy = __fadd_rn(f.gy, fl.y); f.gz = __fadd_rn(f.gz, fl.z);
    }
    const Philox4 xr = philox4x32_10(orig, r, sw_lo, sw_hi, a.key0, a.key1);
    trial_spin(a.mode, a.tilt, st->mag[at], ox, oy, oz, xr.x, xr.y, nx, ny, nz);
    de = delta_energy(hb || a.has_si, f.gx, f.gy, f.gz, f.qxx, f.qyy, f.qzz, f.qxy, f.qxz, f.qyz, ox, oy, oz, nx,
                      ny, nz);
    return metropolis_accept(beta, de, xr.z);
}

__global__ void __launch_bounds__(kTileThreads, 2) k_sweep_tile(const TileArgs a)
{
    const int T = a.T, B = a.T + 2, G = a.G, na = a.na;
    const int ngroups = a.R / G;
    const int group = blockIdx.x % ngroups;
    const int tp = blockIdx.x / ngroups;
    const int hx_t = a.ntx >> 1, hy_t = a.nty >> 1;
    const int tx = 2 * (tp % hx_t) + (a.phase & 1);
    const int ty = 2 * ((tp / hx_t) % hy_t) + ((a.phase >> 1) & 1);
    const int tz = 2 * (tp / (hx_t * hy_t)) + ((a.phase >> 2) & 1);
    const int x0 = tx * T, y0 = ty * T, z0 = tz * T;
    const int r0 = group * G;
    const unsigned long long sweep = a.sweep + (a.ctr ? *a.ctr : 0ull);
    const uint32_t sw_lo = (uint32_t)sweep, sw_hi = (uint32_t)(sweep >> 32);

    // shared memory: stencil header | couplings per (atom, entry) | entry
    // offsets | spins [3][box sites][G]; the reduction scratch reuses the
    // spins after the write-back
    extern __shared__ __align__(16) unsigned char smem[];
    const int maxst = a.maxst;
    ClusterStencil *st = reinterpret_cast<ClusterStencil *>(smem);
    ClusterNbr *nbt = reinterpret_cast<ClusterNbr *>(st + 1);          // [na][maxst]
    int *toff = reinterpret_cast<int *>(nbt + na * maxst);
    const int nbox = B * B * B * na;
    float *sx = reinterpret_cast<float *>(toff + ((na * maxst + 3) & ~3));
    float *sy = sx + (size_t)nbox * G;
    float *sz = sy + (size_t)nbox * G;
    double *red = reinterpret_cast<double *>(sx);                      // [4][kTileThreads], after the write-back
    unsigned long long *red_n = reinterpret_cast<unsigned long long *>(red + 4 * kTileThreads);

    __shared__ int s_nbd8[kMaxClusterAtoms], s_nall8[kMaxClusterAtoms];
    {
        const int *src = reinterpret_cast<const int *>(a.stencil);
        int *dst = reinterpret_cast<int *>(st);
        for (int i = threadIdx.x; i < (int)(sizeof(ClusterStencil) / 4); i += blockDim.x) dst[i] = src[i];
        // couplings and box-site offsets of entry e of atom at:
        // (((dz*B + dy)*B + dx)*na + b) - at
        for (int i = threadIdx.x; i < na * maxst; i += blockDim.x) {
            const int at = i / maxst;
            nbt[i] = a.cpl[i];
            const int4 d = a.offs[i];
            toff[i] = ((d.z * B + d.y) * B + d.x) * na + d.w - at;
        }
        if (threadIdx.x < kMaxClusterAtoms) {
            s_nbd8[threadIdx.x] = a.nbd8[threadIdx.x];
            s_nall8[threadIdx.x] = a.nall8[threadIdx.x];
        }
    }
    // the box: tile + one cell of halo, periodic
    for (int i = threadIdx.x; i < nbox * G; i += blockDim.x) {
        const int g = i % G, bs = i / G;
        const int at = bs % na, cell = bs / na;
        const int bx = cell % B, by = (cell / B) % B, bz = cell / (B * B);
        int x = x0 - 1 + bx, y = y0 - 1 + by, z = z0 - 1 + bz;
        x += (x < 0) ? a.Lx : (x >= a.Lx ? -a.Lx : 0);
        y += (y < 0) ? a.Ly : (y >= a.Ly ? -a.Ly : 0);
        z += (z < 0) ? a.Lz : (z >= a.Lz ? -a.Lz : 0);
        const int orig = ((z * a.Ly + y) * a.Lx + x) * na + at;
        const size_t gi = (size_t)__ldg(a.inv + orig) * a.R + r0 + g;
        sx[i] = a.sx[gi]; sy[i] = a.sy[gi]; sz[i] = a.sz[gi];
    }
    __syncthreads();

    // every item of this thread belongs to replica r0 + (threadIdx.x % G)
    const int g = threadIdx.x % G;
    const int r = r0 + g;
    const float beta = a.beta[a.temp_of[r]];
    float accE = 0.f, accX = 0.f, accY = 0.f, accZ = 0.f;
    unsigned int nrej = 0;
    const int h = T >> 1, per_class = h * h * h;
    for (int c = 0; c < st->ncolour; ++c) {
        const int c0 = st->colour_start[c];
        const int items = (st->colour_start[c + 1] - c0) * per_class * G;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int si = it / G;
            const int k = st->class_order[c0 + si / per_class];
            const int rem = si % per_class;
            const int hx = rem % h, hy = (rem / h) % h, hz = rem / (h * h);
            const int at = k >> 3;
            const int lx = 2 * hx + ((k >> 2) & 1), ly = 2 * hy + ((k >> 1) & 1), lz = 2 * hz + (k & 1);
            const int bsite = (((lz + 1) * B + (ly + 1)) * B + (lx + 1)) * na + at;
            const int l = bsite * G + g;
            const float ox = sx[l], oy = sy[l], oz = sz[l];
            FieldQ f{};
            const ClusterNbr *nb = nbt + at * maxst;
            const int *to = toff + at * maxst;
            const int nbd8 = s_nbd8[at], nall8 = s_nall8[at];
            int e0 = 0;
            for (; e0 < nbd8; e0 += 8) {
                float tx_[8], ty_[8], tz_[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int q = (bsite + to[e0 + j]) * G + g;
                    tx_[j] = sx[q]; ty_[j] = sy[q]; tz_[j] = sz[q];
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const ClusterNbr &se = nb[e0 + j];
                    entry_exchange(f, -se.J, tx_[j], ty_[j], tz_[j]);
                    if (a.has_b) entry_bq(f, se.B, tx_[j], ty_[j], tz_[j]);
                    if (a.has_d) entry_dm(f, se.Dx, se.Dy, se.Dz, tx_[j], ty_[j], tz_[j]);
                }
            }
            for (; e0 < nall8; e0 += 8) {   // exchange only
                float tx_[8], ty_[8], tz_[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int q = (bsite + to[e0 + j]) * G + g;
                    tx_[j] = sx[q]; ty_[j] = sy[q]; tz_[j] = sz[q];
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) entry_exchange(f, -nb[e0 + j].J, tx_[j], ty_[j], tz_[j]);
            }
            const int orig = (((z0 + lz) * a.Ly + (y0 + ly)) * a.Lx + (x0 + lx)) * na + at;
            float nx, ny, nz, de;
            if (tile_trial(a, st, f, at, (uint32_t)orig, (uint32_t)r, sw_lo, sw_hi, beta, ox, oy, oz, nx, ny, nz, de,
                           a.has_b)) {
                sx[l] = nx; sy[l] = ny; sz[l] = nz;
                accE += de;
                accX += __fsub_rn(nx, ox); accY += __fsub_rn(ny, oy); accZ += __fsub_rn(nz, oz);
            } else {
                ++nrej;
            }
        }
        __syncthreads();
    }
    // the tile (not the halo) back to global memory
    const int ntile = T * T * T * na;
    for (int i = threadIdx.x; i < ntile * G; i += blockDim.x) {
        const int gg = i % G, ts = i / G;
        const int at = ts % na, cell = ts / na;
        const int lx = cell % T, ly = (cell / T) % T, lz = cell / (T * T);
        const int bsite = (((lz + 1) * B + (ly + 1)) * B + (lx + 1)) * na + at;
        const int orig = (((z0 + lz) * a.Ly + (y0 + ly)) * a.Lx + (x0 + lx)) * na + at;
        const size_t gi = (size_t)__ldg(a.inv + orig) * a.R + r0 + gg;
        const int l = bsite * G + gg;
        a.sx[gi] = sx[l]; a.sy[gi] = sy[l]; a.sz[gi] = sz[l];
    }
    // per-replica sums of this tile, in a fixed order, into the tile's slots
    __syncthreads();   // the spins are written back; their space becomes the scratch
    red[threadIdx.x] = (double)accE;
    red[kTileThreads + threadIdx.x] = (double)accX;
    red[2 * kTileThreads + threadIdx.x] = (double)accY;
    red[3 * kTileThreads + threadIdx.x] = (double)accZ;
    red_n[threadIdx.x] = nrej;
    __syncthreads();
    if ((int)threadIdx.x < G) {
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        unsigned long long sn = 0;
        for (int t = threadIdx.x; t < (int)blockDim.x; t += G) {
            s0 += red[t]; s1 += red[kTileThreads + t]; s2 += red[2 * kTileThreads + t]; s3 += red[3 * kTileThreads + t];
            sn += red_n[t];
        }
        const int tile = (tz * a.nty + ty) * a.ntx + tx;
        const size_t slot = (size_t)tile * a.R + r0 + threadIdx.x;
        double *o = a.part + 4 * slot;
        o[0] += s0; o[1] += s1; o[2] += s2; o[3] += s3;
        a.part_rej[slot] += sn;
    }
}

// ---------------------------------------------------------------------------
// Pipelined variant: persistent CTAs of 256 threads, one per SM, loop over the
// (tile, replica group) items of the launch's tile parity.  While item k is
// updated in one shared-memory buffer, the box of item k+1 arrives in the
// other by cp.async (16-byte chunks: the G replicas of a site are contiguous)
// and the site-index lookups of item k+2 are in flight in registers.  Tile
// edge T and group size G are compile-time constants.  A thread updates two
// replicas of a site: each neighbour costs one slot lookup and three 8-byte
// shared-memory loads (x, y, z of both replicas sit in one slot), and the
// field sums run as fma.rn.f32x2 on the pair.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Shared-memory slot of box site b: within each block of 8 sites,
// b = 8 blk + 2 a + p goes to slot 8 blk + a + 4 p, so sites two apart (one
// colour class along x: the 4 sites one warp reads with 8 replicas each) land
// in 4 distinct 8-bank groups.
__device__ __forceinline__ int box_slot(int b) { return (b & ~7) | ((b >> 1) & 3) | ((b & 1) << 2); }

constexpr int kTilePThreads = 256;
// threads of a persistent CTA: 128 for groups of 4 replicas with one box
// buffer (four CTAs per SM: the same warps per SM as two of 256, in items of
// half the size, so a launch's last round idles less), else 256
__host__ __device__ constexpr int tile_p_nt(int G, int NB) { return NB == 1 && G == 4 ? 128 : kTilePThreads; }
constexpr int kInvPerThread = 16;   // box sites per thread for the index prefetch (<= 4096 box sites)

// Couplings of one stencil entry with every value in both lanes of a float2,
// for the two-replica arithmetic: -J, B, D and -D.
struct PairNbr {
    float2 nJ, B, Dx, Dy, Dz, nDx, nDy, nDz;
};

// NB box buffers per CTA.  NB = 2: one CTA per SM, the next item's box copied
// while this one's sites are updated.  NB = 1: two CTAs per SM at <= 128
// registers a thread, twice the warps; each CTA copies its box, then updates,
// and the other CTA's updates cover the copy.  EG stencil entries per group
// of neighbour loads in flight.
// FL: the biquadratic (bit 0) and DM (bit 1) terms as compile-time flags, or
// 4: read from the arguments (the one-CTA-per-SM variant, kept to one
// instantiation per shape).
template <int T, int G, int NB, int FL>
__global__ void __launch_bounds__(tile_p_nt(G, NB), NB == 2 ? 1 : 2 * kTilePThreads / tile_p_nt(G, NB))
    k_sweep_tile_p(const TileArgs a)
{
    // SL floats per box slot: x of the G replicas, then y, then z; a thread
    // updates replicas (2 gp, 2 gp + 1) of a site
    constexpr int NT = tile_p_nt(G, NB), B = T + 2, H = T / 2, PC = H * H * H, CH = G / 4, GP = G / 2, SL = 3 * G;
    // entries per group of neighbour loads in flight: B/DM entries (EB), then
    // exchange-only ones (EG); the bounds skip the table's padding beyond them
    constexpr int EB = NB == 2 ? 8 : 2, EG = NB == 2 ? 8 : 4;
    static_assert(NB == 1 || NB == 2, "box buffers");
    const bool hb = FL == 4 ? a.has_b != 0 : (FL & 1) != 0;
    const bool hd = FL == 4 ? a.has_d != 0 : (FL & 2) != 0;
    static_assert(G % 4 == 0 && 32 % GP == 0 && (T & 1) == 0, "tile shape");
    const int na = a.na, maxst = a.maxst;
    const int ngroups = a.R / G;
    const int hx_t = a.ntx >> 1, hy_t = a.nty >> 1, hz_t = a.ntz >> 1;
    const int W = hx_t * hy_t * hz_t * ngroups;
    const int nbs = B * B * B * na;
    const int nbs8 = (nbs + 7) & ~7;   // box sites rounded to whole slot blocks
    const unsigned long long sweep = a.sweep + (a.ctr ? *a.ctr : 0ull);
    const uint32_t sw_lo = (uint32_t)sweep, sw_hi = (uint32_t)(sweep >> 32);

    extern __shared__ __align__(16) unsigned char smem[];
    ClusterStencil *st = reinterpret_cast<ClusterStencil *>(smem);
    PairNbr *pnb = reinterpret_cast<PairNbr *>(st + 1);                // [na][maxst]
    // slot offsets (in floats) of the entries for each value of (box site & 7):
    // box_slot(b + o) - box_slot(b) depends on o and b & 7 only
    int *tq = reinterpret_cast<int *>(pnb + na * maxst);                // [na][maxst][8]
    int *inv_s = tq + 8 * na * maxst;                                   // [NB][nbs], padded to 4
    float *buf = reinterpret_cast<float *>(inv_s + NB * ((nbs + 3) & ~3));  // [NB][nbs8][3][G]
    double *red = reinterpret_cast<double *>(buf + (size_t)NB * nbs8 * SL);  // [NT/32][G][4]
    unsigned long long *red_n = reinterpret_cast<unsigned long long *>(red + (NT / 32) * G * 4);

    __shared__ int s_nbd8[kMaxClusterAtoms], s_nall8[kMaxClusterAtoms];
    __shared__ int s_nbd2[kMaxClusterAtoms], s_nall4[kMaxClusterAtoms];
    {
        const int *src = reinterpret_cast<const int *>(a.stencil);
        int *dst = reinterpret_cast<int *>(st);
        for (int i = threadIdx.x; i < (int)(sizeof(ClusterStencil) / 4); i += NT) dst[i] = src[i];
        for (int i = threadIdx.x; i < na * maxst; i += NT) {
            const int at = i / maxst;
            const ClusterNbr c = a.cpl[i];
            PairNbr p;
            p.nJ = make_float2(-c.J, -c.J); p.B = make_float2(c.B, c.B);
            p.Dx = make_float2(c.Dx, c.Dx); p.Dy = make_float2(c.Dy, c.Dy); p.Dz = make_float2(c.Dz, c.Dz);
            p.nDx = make_float2(-c.Dx, -c.Dx); p.nDy = make_float2(-c.Dy, -c.Dy); p.nDz = make_float2(-c.Dz, -c.Dz);
            pnb[i] = p;
            const int4 d = a.offs[i];
            const int o = ((d.z * B + d.y) * B + d.x) * na + d.w - at;
            for (int m = 0; m < 8; ++m) {
                const int b = (1 << 20) + m;   // any box site with b & 7 == m
                tq[8 * i + m] = (box_slot(b + o) - box_slot(b)) * SL;
            }
        }
        if (threadIdx.x < kMaxClusterAtoms) {
            s_nbd8[threadIdx.x] = a.nbd8[threadIdx.x];
            s_nall8[threadIdx.x] = a.nall8[threadIdx.x];
            s_nbd2[threadIdx.x] = a.nbd2[threadIdx.x];
            s_nall4[threadIdx.x] = a.nall4[threadIdx.x];
        }
    }

    // item -> tile origin and first replica
    auto item_tile = [&](int w, int &x0, int &y0, int &z0, int &r0, int &tile) {
        const int tp = w / ngroups;
        r0 = (w % ngroups) * G;
        const int tx = 2 * (tp % hx_t) + (a.phase & 1);
        const int ty = 2 * ((tp / hx_t) % hy_t) + ((a.phase >> 1) & 1);
        const int tz = 2 * (tp / (hx_t * hy_t)) + ((a.phase >> 2) & 1);
        x0 = tx * T; y0 = ty * T; z0 = tz * T;
        tile = (tz * a.nty + ty) * a.ntx + tx;
    };
    // reference-site index -> permuted index of the box sites of item w
    auto load_inv = [&](int w, int (&regs)[kInvPerThread]) {
        int x0, y0, z0, r0, tile;
        item_tile(w, x0, y0, z0, r0, tile);
#pragma unroll
        for (int j = 0; j < kInvPerThread; ++j) {
            const int i = threadIdx.x + j * NT;
            int v = 0;
            if (i < nbs) {
                const int at = na == 1 ? 0 : i % na, cell = na == 1 ? i : i / na;
                const int bx = cell % B, by = (cell / B) % B, bz = cell / (B * B);
                int x = x0 - 1 + bx, y = y0 - 1 + by, z = z0 - 1 + bz;
                x += (x < 0) ? a.Lx : (x >= a.Lx ? -a.Lx : 0);
                y += (y < 0) ? a.Ly : (y >= a.Ly ? -a.Ly : 0);
                z += (z < 0) ? a.Lz : (z >= a.Lz ? -a.Lz : 0);
                v = __ldg(a.inv + ((z * a.Ly + y) * a.Lx + x) * na + at);
            }
            regs[j] = v;
        }
    };
    auto store_inv = [&](int stage, const int (&regs)[kInvPerThread]) {
#pragma unroll
        for (int j = 0; j < kInvPerThread; ++j) {
            const int i = threadIdx.x + j * NT;
            if (i < nbs) inv_s[stage * ((nbs + 3) & ~3) + i] = regs[j];
        }
    };
    // the box of item w into buffer `stage`, as 16-byte asynchronous copies:
    // chunk k of a box site is component k / CH, replicas 4 (k % CH) ..
    auto issue_box = [&](int w, int stage) {
        int x0, y0, z0, r0, tile;
        item_tile(w, x0, y0, z0, r0, tile);
        const int *inv = inv_s + stage * ((nbs + 3) & ~3);
        float *dst = buf + (size_t)stage * nbs8 * SL;
        for (int i = threadIdx.x; i < nbs * 3 * CH; i += NT) {
            const int k = i % (3 * CH), bs = i / (3 * CH);
            const int cp = k / CH, c = k % CH;
            const float *base = cp == 0 ? a.sx : (cp == 1 ? a.sy : a.sz);
            const float *src = base + (size_t)inv[bs] * a.R + r0 + 4 * c;
            cp_async16(dst + box_slot(bs) * SL + 4 * k, src);
        }
        cp_async_commit();
    };

    int w = blockIdx.x;
    if (w >= W) return;
    int regs[kInvPerThread];
    if constexpr (NB == 2) {
        load_inv(w, regs);
        store_inv(0, regs);
        __syncthreads();
        issue_box(w, 0);
        const int w1 = w + gridDim.x;
        if (w1 < W) {
            load_inv(w1, regs);
            store_inv(1, regs);
        }
    }
    const int gp = threadIdx.x % GP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int kk = 0; w < W; ++kk, w += gridDim.x) {
        const int cur = NB == 2 ? (kk & 1) : 0;
        const int wn = w + gridDim.x, wnn = wn + gridDim.x;
        if constexpr (NB == 2) {
            __syncthreads();   // inv_s[nxt] written, buffer nxt free
            if (wn < W) issue_box(wn, cur ^ 1);
            if (wnn < W) load_inv(wnn, regs);   // in flight during the update
            if (wn < W) cp_async_wait<1>(); else cp_async_wait<0>();
        } else {
            // the previous item's write-back and sums are done (barrier at
            // the end of the loop body): its index table and box are free
            load_inv(w, regs);
            store_inv(0, regs);
            __syncthreads();
            issue_box(w, 0);
            cp_async_wait<0>();
        }
        __syncthreads();   // box of item w visible to every thread

        int x0, y0, z0, r0, tile;
        item_tile(w, x0, y0, z0, r0, tile);
        float *sb = buf + (size_t)cur * nbs8 * SL;
        const int r = r0 + 2 * gp;
        const float beta0 = a.beta[a.temp_of[r]], beta1 = a.beta[a.temp_of[r + 1]];
        float accE[2] = {0.f, 0.f}, accX[2] = {0.f, 0.f}, accY[2] = {0.f, 0.f}, accZ[2] = {0.f, 0.f};
        unsigned int nrej[2] = {0u, 0u};
        for (int c = 0; c < st->ncolour; ++c) {
            const int c0 = st->colour_start[c];
            const int items = (st->colour_start[c + 1] - c0) * PC * GP;
            for (int it = threadIdx.x; it < items; it += NT) {
                const int si = it / GP;
                const int kcl = st->class_order[c0 + si / PC];
                const int rem = si % PC;
                const int hx = rem % H, hy = (rem / H) % H, hz = rem / (H * H);
                const int at = kcl >> 3;
                const int lx = 2 * hx + ((kcl >> 2) & 1), ly = 2 * hy + ((kcl >> 1) & 1), lz = 2 * hz + (kcl & 1);
                const int bsite = (((lz + 1) * B + (ly + 1)) * B + (lx + 1)) * na + at;
                float *own = sb + box_slot(bsite) * SL + 2 * gp;
                const float2 ox = *reinterpret_cast<const float2 *>(own);
                const float2 oy = *reinterpret_cast<const float2 *>(own + G);
                const float2 oz = *reinterpret_cast<const float2 *>(own + 2 * G);
                FieldQ2 f;
                f.gx = f.gy = f.gz = f.qxx = f.qyy = f.qzz = f.qxy = f.qxz = f.qyz = make_float2(0.f, 0.f);
                const PairNbr *nb = pnb + at * maxst;
                const int *to = tq + 8 * at * maxst + (bsite & 7);
                const int nbd = NB == 2 ? s_nbd8[at] : s_nbd2[at];
                const int nall = NB == 2 ? s_nall8[at] : s_nall4[at];
                int e0 = 0;
                for (; e0 < nbd; e0 += EB) {
                    float2 tx_[EB], ty_[EB], tz_[EB];
#pragma unroll
                    for (int j = 0; j < EB; ++j) {
                        const float *q = own + to[8 * (e0 + j)];
                        tx_[j] = *reinterpret_cast<const float2 *>(q);
                        ty_[j] = *reinterpret_cast<const float2 *>(q + G);
                        tz_[j] = *reinterpret_cast<const float2 *>(q + 2 * G);
                    }
#pragma unroll
                    for (int j = 0; j < EB; ++j) {
                        const PairNbr &p = nb[e0 + j];
                        entry_exchange(f, p.nJ, tx_[j], ty_[j], tz_[j]);
                        if (hb) entry_bq(f, p.B, tx_[j], ty_[j], tz_[j]);
                        if (hd) entry_dm(f, p.Dx, p.Dy, p.Dz, p.nDx, p.nDy, p.nDz, tx_[j], ty_[j], tz_[j]);
                    }
                }
                for (e0 = s_nbd8[at]; e0 < nall; e0 += EG) {   // exchange only
                    float2 tx_[EG], ty_[EG], tz_[EG];
#pragma unroll
                    for (int j = 0; j < EG; ++j) {
                        const float *q = own + to[8 * (e0 + j)];
                        tx_[j] = *reinterpret_cast<const float2 *>(q);
                        ty_[j] = *reinterpret_cast<const float2 *>(q + G);
                        tz_[j] = *reinterpret_cast<const float2 *>(q + 2 * G);
                    }
#pragma unroll
                    for (int j = 0; j < EG; ++j) entry_exchange(f, nb[e0 + j].nJ, tx_[j], ty_[j], tz_[j]);
                }
                const int orig = (((z0 + lz) * a.Ly + (y0 + ly)) * a.Lx + (x0 + lx)) * na + at;
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const float sx0 = k ? ox.y : ox.x, sy0 = k ? oy.y : oy.x, sz0 = k ? oz.y : oz.x;
                    float nx, ny, nz, de;
                    if (tile_trial(a, st, lane_of(f, k), at, (uint32_t)orig, (uint32_t)(r + k), sw_lo, sw_hi,
                                   k ? beta1 : beta0, sx0, sy0, sz0, nx, ny, nz, de, hb)) {
                        own[k] = nx; own[G + k] = ny; own[2 * G + k] = nz;
                        accE[k] += de;
                        accX[k] += __fsub_rn(nx, sx0); accY[k] += __fsub_rn(ny, sy0); accZ[k] += __fsub_rn(nz, sz0);
                    } else {
                        ++nrej[k];
                    }
                }
            }
            __syncthreads();
        }
        // write the tile back (16-byte chunks), its sums to the tile's slots
        {
            const int *inv = inv_s + cur * ((nbs + 3) & ~3);
            for (int i = threadIdx.x; i < T * T * T * na * 3 * CH; i += NT) {
                const int k = i % (3 * CH), ts = i / (3 * CH);
                const int cp = k / CH, c = k % CH;
                const int at = na == 1 ? 0 : ts % na, cell = na == 1 ? ts : ts / na;
                const int lx = cell % T, ly = (cell / T) % T, lz = cell / (T * T);
                const int bsite = (((lz + 1) * B + (ly + 1)) * B + (lx + 1)) * na + at;
                const float4 v = *reinterpret_cast<const float4 *>(sb + box_slot(bsite) * SL + 4 * k);
                float *base = cp == 0 ? a.sx : (cp == 1 ? a.sy : a.sz);
                *reinterpret_cast<float4 *>(base + (size_t)inv[bsite] * a.R + r0 + 4 * c) = v;
            }
        }
        // lanes with the same gp hold the same two replicas
        double v[2][4];
        unsigned long long nr[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            v[k][0] = accE[k]; v[k][1] = accX[k]; v[k][2] = accY[k]; v[k][3] = accZ[k];
            nr[k] = nrej[k];
        }
        for (int o = GP; o < 32; o <<= 1) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                for (int q = 0; q < 4; ++q) v[k][q] += __shfl_xor_sync(0xffffffffu, v[k][q], o);
                nr[k] += __shfl_xor_sync(0xffffffffu, nr[k], o);
            }
        }
        if (lane < GP) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                for (int q = 0; q < 4; ++q) red[(warp * G + 2 * lane + k) * 4 + q] = v[k][q];
                red_n[warp * G + 2 * lane + k] = nr[k];
            }
        }
        __syncthreads();   // sums in place; nobody reads inv_s[cur] any more
        if ((int)threadIdx.x < G) {
            double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            unsigned long long sn = 0;
            for (int q = 0; q < NT / 32; ++q) {
                const double *o = red + (q * G + threadIdx.x) * 4;
                s0 += o[0]; s1 += o[1]; s2 += o[2]; s3 += o[3];
                sn += red_n[q * G + threadIdx.x];
            }
            const size_t slot = (size_t)tile * a.R + r0 + threadIdx.x;
            double *o = a.part + 4 * slot;
            o[0] += s0; o[1] += s1; o[2] += s2; o[3] += s3;
            a.part_rej[slot] += sn;
        }
        if constexpr (NB == 2) {
            if (wnn < W) store_inv(cur, regs);
        }
    }
}

// e_run / m_run / rejected of every replica from the tiles' slots, and the
// slots cleared, in two passes with a fixed summation order (deterministic
// for any grid).  Pass 1: block (b, y) sums tiles [32 b, 32 b + 32) of slot
// words [256 y, 256 y + 256), thread q of the words (4 R doubles, then R
// counts) walking the tiles in order, so a warp reads 32 consecutive words of
// a tile.
__global__ void __launch_bounds__(256) k_tile_fold_chunks(TileFoldArgs a)
{
    const int t0 = blockIdx.x * kTileFoldChunk;
    const int t1 = min(a.ntiles, t0 + kTileFoldChunk);
    const int W = 4 * a.R;
    double *chunk = a.part + (size_t)a.ntiles * W;
    unsigned long long *chunk_rej = a.part_rej + (size_t)a.ntiles * a.R;
    const int q = blockIdx.y * blockDim.x + threadIdx.x;
    if (q < W + a.R) {
        // loads first, then the clearing stores, so the loads of a thread
        // are all in flight together
        if (q < W) {
            double *o = a.part + (size_t)t0 * W + q;
            double s = 0.0;
#pragma unroll 8
            for (int k = 0; k < t1 - t0; ++k) s += o[(size_t)k * W];
            for (int k = 0; k < t1 - t0; ++k) o[(size_t)k * W] = 0.0;
            chunk[(size_t)blockIdx.x * W + q] = s;
        } else {
            unsigned long long *o = a.part_rej + (size_t)t0 * a.R + (q - W);
            unsigned long long n = 0;
#pragma unroll 8
            for (int k = 0; k < t1 - t0; ++k) n += o[(size_t)k * a.R];
            for (int k = 0; k < t1 - t0; ++k) o[(size_t)k * a.R] = 0ull;
            chunk_rej[(size_t)blockIdx.x * a.R + (q - W)] = n;
        }
    }
}

// Pass 2: thread q sums slot word q over the chunks in order.
__global__ void __launch_bounds__(256) k_tile_fold_total(TileFoldArgs a)
{
    const int W = 4 * a.R, nch = tile_fold_chunks(a.ntiles);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const double *chunk = a.part + (size_t)a.ntiles * W;
    const unsigned long long *chunk_rej = a.part_rej + (size_t)a.ntiles * a.R;
    if (q < W) {
        double s = 0.0;
        for (int b = 0; b < nch; ++b) s += chunk[(size_t)b * W + q];
        const int r = q >> 2, c = q & 3;
        if (c == 0) a.e_run[r] += s;
        else a.m_run[3 * r + c - 1] += s;
    } else if (q < W + a.R) {
        const int r = q - W;
        unsigned long long n = 0;
        for (int b = 0; b < nch; ++b) n += chunk_rej[(size_t)b * a.R + r];
        a.rej[2 * a.temp_of[r] + a.phase] += n;
    }
}

}  // namespace

size_t tile_smem_bytes(int T, int G, int na, int maxst)
{
    const size_t B = (size_t)T + 2;
    const size_t spins = (size_t)3 * B * B * B * na * G * sizeof(float);
    const size_t scratch = (size_t)kTileThreads * (4 * sizeof(double) + sizeof(unsigned long long));
    return sizeof(ClusterStencil) + (size_t)na * maxst * sizeof(ClusterNbr) +
           (size_t)((na * maxst + 3) & ~3) * sizeof(int) + (spins > scratch ? spins : scratch);
}

cudaError_t tile_configure(size_t smem)
{
    return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sweep_tile), smem);
}

cudaError_t launch_tile(const TileArgs &a, size_t smem, cudaStream_t st)
{
    if (a.G <= 0 || a.R % a.G != 0 || kTileThreads % a.G != 0 || (a.T & 1) || a.T <= 0) return cudaErrorInvalidValue;
    const int tiles = (a.ntx / 2) * (a.nty / 2) * (a.ntz / 2);
    k_sweep_tile<<<tiles * (a.R / a.G), kTileThreads, smem, st>>>(a);
    return cudaGetLastError();
}

size_t tile_p_smem_bytes(int T, int G, int na, int maxst, int nb)
{
    const size_t B = (size_t)T + 2, nbs = B * B * B * na, nbs8 = (nbs + 7) & ~(size_t)7;
    return sizeof(ClusterStencil) + (size_t)na * maxst * sizeof(PairNbr) +
           (size_t)8 * na * maxst * sizeof(int) + nb * ((nbs + 3) & ~(size_t)3) * sizeof(int) +
           (size_t)3 * nb * nbs8 * G * sizeof(float) + (size_t)(tile_p_nt(G, nb) / 32) * G * (4 * sizeof(double) + 8);
}

bool tile_p_supported(int T, int G, int na)
{
    const int B = T + 2;
    if (B * B * B * na > kInvPerThread * tile_p_nt(G, 1)) return false;   // the smaller CTA bounds it
    return (T == 4 || T == 6 || T == 8) && (G == 4 || G == 8 || G == 16);
}

namespace {
// configure: allow the shared memory; blocks < 0: store the CTAs one SM
// holds in *per_sm (the occupancy calculator); else launch `blocks` CTAs
template <int T, int G, int NB, int FL>
cudaError_t launch_pf(const TileArgs &a, size_t smem, int blocks, cudaStream_t st, bool configure,
                      int *per_sm = nullptr)
{
    if (configure) return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sweep_tile_p<T, G, NB, FL>), smem);
    if (blocks < 0)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_sweep_tile_p<T, G, NB, FL>, tile_p_nt(G, NB),
                                                             smem);
    k_sweep_tile_p<T, G, NB, FL><<<blocks, tile_p_nt(G, NB), smem, st>>>(a);
    return cudaGetLastError();
}

// the two-CTA variant with the terms as compile-time flags (configured all
// four at once), the one-CTA variant reading them from the arguments
template <int T, int G, int NB>
cudaError_t launch_p(const TileArgs &a, size_t smem, int blocks, cudaStream_t st, bool configure, int *per_sm)
{
    if constexpr (NB == 2) {
        return launch_pf<T, G, NB, 4>(a, smem, blocks, st, configure, per_sm);
    } else {
        if (configure) {
            cudaError_t e = launch_pf<T, G, NB, 0>(a, smem, blocks, st, true);
            if (e == cudaSuccess) e = launch_pf<T, G, NB, 1>(a, smem, blocks, st, true);
            if (e == cudaSuccess) e = launch_pf<T, G, NB, 2>(a, smem, blocks, st, true);
            if (e == cudaSuccess) e = launch_pf<T, G, NB, 3>(a, smem, blocks, st, true);
            return e;
        }
        switch ((a.has_b ? 1 : 0) | (a.has_d ? 2 : 0)) {
        case 0: return launch_pf<T, G, NB, 0>(a, smem, blocks, st, false, per_sm);
        case 1: return launch_pf<T, G, NB, 1>(a, smem, blocks, st, false, per_sm);
        case 2: return launch_pf<T, G, NB, 2>(a, smem, blocks, st, false, per_sm);
        default: return launch_pf<T, G, NB, 3>(a, smem, blocks, st, false, per_sm);
        }
    }
}

template <int T, int NB>
cudaError_t launch_pg(const TileArgs &a, size_t smem, int blocks, cudaStream_t st, bool configure, int *per_sm)
{
    if (a.G == 4) return launch_p<T, 4, NB>(a, smem, blocks, st, configure, per_sm);
    if (a.G == 8) return launch_p<T, 8, NB>(a, smem, blocks, st, configure, per_sm);
    if (a.G == 16) return launch_p<T, 16, NB>(a, smem, blocks, st, configure, per_sm);
    return cudaErrorInvalidValue;
}

template <int NB>
cudaError_t launch_pt(const TileArgs &a, size_t smem, int blocks, cudaStream_t st, bool configure,
                      int *per_sm = nullptr)
{
    if (a.T == 4) return launch_pg<4, NB>(a, smem, blocks, st, configure, per_sm);
    if (a.T == 6) return launch_pg<6, NB>(a, smem, blocks, st, configure, per_sm);
    if (a.T == 8) return launch_pg<8, NB>(a, smem, blocks, st, configure, per_sm);
    return cudaErrorInvalidValue;
}
}  // namespace

cudaError_t tile_p_configure(int T, int G, int nb, size_t smem)
{
    TileArgs a{};
    a.T = T; a.G = G;
    if (nb == 1) return launch_pt<1>(a, smem, 0, nullptr, true);
    if (nb == 2) return launch_pt<2>(a, smem, 0, nullptr, true);
    return cudaErrorInvalidValue;
}

cudaError_t tile_p_grid(const TileArgs &a, size_t smem, int num_sms, int nb, int *blocks)
{
    if (!tile_p_supported(a.T, a.G, a.na) || a.R % a.G != 0 || (nb != 1 && nb != 2) || num_sms < 1 || !blocks)
        return cudaErrorInvalidValue;
    int per_sm = 0;
    const cudaError_t e = nb == 1 ? launch_pt<1>(a, smem, -1, nullptr, false, &per_sm)
                                  : launch_pt<2>(a, smem, -1, nullptr, false, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const long long items = (long long)(a.ntx / 2) * (a.nty / 2) * (a.ntz / 2) * (a.R / a.G);
    *blocks = (int)std::min<long long>(items, (long long)per_sm * num_sms);
    return cudaSuccess;
}

cudaError_t launch_tile_p(const TileArgs &a, size_t smem, int blocks, int nb, cudaStream_t st)
{
    if (!tile_p_supported(a.T, a.G, a.na) || a.R % a.G != 0 || (nb != 1 && nb != 2) || blocks < 1)
        return cudaErrorInvalidValue;
    return nb == 1 ? launch_pt<1>(a, smem, blocks, st, false) : launch_pt<2>(a, smem, blocks, st, false);
}

cudaError_t launch_tile_fold(const TileFoldArgs &a, cudaStream_t st)
{
    k_tile_fold_chunks<<<dim3(tile_fold_chunks(a.ntiles), (5 * a.R + 255) / 256), 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_tile_fold_total<<<(5 * a.R + 255) / 256, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace esp
