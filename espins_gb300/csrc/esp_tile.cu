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

namespace esp {

namespace {

constexpr int kTileThreads = 256;

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

    {
        // header, then the entries of class 8*at (every parity class of an
        // atom has the same couplings)
        const int *src = reinterpret_cast<const int *>(a.stencil);
        int *dst = reinterpret_cast<int *>(st);
        for (int i = threadIdx.x; i < (int)(sizeof(ClusterStencil) / 4); i += blockDim.x) dst[i] = src[i];
        const ClusterNbr *gn = reinterpret_cast<const ClusterNbr *>(a.stencil + 1);
        for (int i = threadIdx.x; i < na * maxst; i += blockDim.x) {
            const int at = i / maxst, e = i % maxst;
            nbt[i] = gn[(size_t)(8 * at) * maxst + e];
        }
        // box-site offset of entry e of atom at: (((dz*B + dy)*B + dx)*na + b) - at; 0 (the
        // site itself, zero couplings) for padding entries
        for (int i = threadIdx.x; i < na * maxst; i += blockDim.x) {
            const int at = i / maxst, e = i % maxst;
            int o = 0;
            if (e < a.count[at]) {
                const int4 d = a.offs[i];
                o = ((d.z * B + d.y) * B + d.x) * na + d.w - at;
            }
            toff[i] = o;
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
            float gx = 0.f, gy = 0.f, gz = 0.f;
            float qxx = 0.f, qyy = 0.f, qzz = 0.f, qxy = 0.f, qxz = 0.f, qyz = 0.f;
            const int ne8 = (st->count[k] + 7) & ~7;
            const ClusterNbr *nb = nbt + at * maxst;
            const int *to = toff + at * maxst;
            for (int e0 = 0; e0 < ne8; e0 += 8) {
                float tx_[8], ty_[8], tz_[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int q = (bsite + to[e0 + j]) * G + g;
                    tx_[j] = sx[q]; ty_[j] = sy[q]; tz_[j] = sz[q];
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const ClusterNbr &se = nb[e0 + j];
                    const float J = se.J;
                    gx = fmaf(-J, tx_[j], gx); gy = fmaf(-J, ty_[j], gy); gz = fmaf(-J, tz_[j], gz);
                    if (a.has_b) {
                        const float Bv = se.B;
                        const float bx = Bv * tx_[j], by = Bv * ty_[j], bz = Bv * tz_[j];
                        qxx = fmaf(bx, tx_[j], qxx); qyy = fmaf(by, ty_[j], qyy); qzz = fmaf(bz, tz_[j], qzz);
                        qxy = fmaf(bx, ty_[j], qxy); qxz = fmaf(bx, tz_[j], qxz); qyz = fmaf(by, tz_[j], qyz);
                    }
                    if (a.has_d) {
                        const float dx = se.Dx, dy = se.Dy, dz = se.Dz;
                        gx += ty_[j] * dz - tz_[j] * dy;
                        gy += tz_[j] * dx - tx_[j] * dz;
                        gz += tx_[j] * dy - ty_[j] * dx;
                    }
                }
            }
            if (a.has_si) {
                const float4 s = st->si[at];
                const float dx = s.w * s.x, dy = s.w * s.y, dz = s.w * s.z;
                qxx = fmaf(dx, s.x, qxx); qyy = fmaf(dy, s.y, qyy); qzz = fmaf(dz, s.z, qzz);
                qxy = fmaf(dx, s.y, qxy); qxz = fmaf(dx, s.z, qxz); qyz = fmaf(dy, s.z, qyz);
            }
            if (a.has_f) {
                const float4 f = st->fld[at];
                gx += f.x; gy += f.y; gz += f.z;
            }
            const int orig = (((z0 + lz) * a.Ly + (y0 + ly)) * a.Lx + (x0 + lx)) * na + at;
            const Philox4 xr = philox4x32_10((uint32_t)orig, (uint32_t)r, sw_lo, sw_hi, a.key0, a.key1);
            float nx, ny, nz;
            trial_spin(a.mode, a.tilt, st->mag[at], ox, oy, oz, xr.x, xr.y, nx, ny, nz);
            const float dx = nx - ox, dy = ny - oy, dz = nz - oz;
            float de = gx * dx + gy * dy + gz * dz;
            if (a.has_b || a.has_si) {
                const float px2 = nx + ox, py2 = ny + oy, pz2 = nz + oz;
                de += dx * (qxx * px2 + qxy * py2 + qxz * pz2)
                    + dy * (qxy * px2 + qyy * py2 + qyz * pz2)
                    + dz * (qxz * px2 + qyz * py2 + qzz * pz2);
            }
            bool acc = true;
            if (de > 0.0f) acc = expf(-beta * de) >= u24f(xr.z);
            if (acc) {
                sx[l] = nx; sy[l] = ny; sz[l] = nz;
                accE += de;
                accX += dx; accY += dy; accZ += dz;
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

// e_run / m_run / rejected of every replica from the tiles' slots, in tile
// order, and the slots cleared.  One block per replica.
__global__ void __launch_bounds__(256) k_tile_fold(TileFoldArgs a)
{
    __shared__ double s_v[4][256];
    __shared__ unsigned long long s_n[256];
    const int r = blockIdx.x, t = threadIdx.x;
    double v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    unsigned long long n = 0;
    for (int tile = t; tile < a.ntiles; tile += blockDim.x) {
        const size_t slot = (size_t)tile * a.R + r;
        double *o = a.part + 4 * slot;
        v0 += o[0]; v1 += o[1]; v2 += o[2]; v3 += o[3];
        o[0] = 0.0; o[1] = 0.0; o[2] = 0.0; o[3] = 0.0;
        n += a.part_rej[slot];
        a.part_rej[slot] = 0ull;
    }
    s_v[0][t] = v0; s_v[1][t] = v1; s_v[2][t] = v2; s_v[3][t] = v3; s_n[t] = n;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) {
            for (int c = 0; c < 4; ++c) s_v[c][t] += s_v[c][t + w];
            s_n[t] += s_n[t + w];
        }
        __syncthreads();
    }
    if (t == 0) {
        a.e_run[r] += s_v[0][0];
        a.m_run[3 * r] += s_v[1][0]; a.m_run[3 * r + 1] += s_v[2][0]; a.m_run[3 * r + 2] += s_v[3][0];
        a.rej[2 * a.temp_of[r] + a.phase] += s_n[0];
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
    return cudaFuncSetAttribute(k_sweep_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_tile(const TileArgs &a, size_t smem, cudaStream_t st)
{
    if (a.G <= 0 || a.R % a.G != 0 || kTileThreads % a.G != 0 || (a.T & 1) || a.T <= 0) return cudaErrorInvalidValue;
    const int tiles = (a.ntx / 2) * (a.nty / 2) * (a.ntz / 2);
    k_sweep_tile<<<tiles * (a.R / a.G), kTileThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_tile_fold(const TileFoldArgs &a, cudaStream_t st)
{
    k_tile_fold<<<a.R, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace esp
