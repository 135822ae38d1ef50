// Host-side preparation of the device tables: merging the reference's three
// ELL tables into one neighbour list per site, colouring the interaction
// graph and ordering the sites colour by colour.
//
// Input layout (ESpinS jij.F90:32-39, bij.F90:32-34, dij.F90:32-34):
// nbors(N,maxnb) column-major with 1-based indices, values(N,maxnb), and
// dij_matrix(3,N,maxnb).
#include "esp_tables.h"

#include <algorithm>
#include <cstring>
#include <numeric>

namespace esp {

namespace {

struct Entry {
    int32_t j;
    double J, B, D[3];
};

// Sequential greedy colouring of a small graph, trying to reach k colours by
// bounded backtracking first (exact for the class graphs of lattices).
bool colour_k(const std::vector<std::vector<char>> &adj, int k, std::vector<int> &col, long long &budget)
{
    const int n = (int)adj.size();
    col.assign(n, -1);
    // order: largest degree first
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::vector<int> deg(n, 0);
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) deg[a] += adj[a][b];
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return deg[a] > deg[b]; });
    std::vector<int> stack_c(n, -1);
    int pos = 0;
    while (pos >= 0 && pos < n) {
        if (--budget < 0) return false;
        const int v = order[pos];
        int c = col[v] + 1;
        for (; c < k; ++c) {
            bool ok = true;
            for (int u = 0; u < n && ok; ++u)
                if (adj[v][u] && col[u] == c) ok = false;
            if (ok) break;
        }
        if (c < k) {
            col[v] = c;
            ++pos;
        } else {
            col[v] = -1;
            --pos;
        }
    }
    return pos == n;
}

}  // namespace

int prepare_tables(const PrepInput &in, PrepOutput &out, std::string &err)
{
    const int N = in.N;
    const int na = in.num_atoms;
    if (N <= 0 || na <= 0 || N % na != 0) { err = "num_sites must be a positive multiple of num_atoms"; return 1; }
    if ((long long)in.L[0] * in.L[1] * in.L[2] * na != N) { err = "num_sites != prod(supercell)*num_atoms"; return 1; }
    if (!in.mag || !in.j_nn || !in.j_nbors || !in.j_val) { err = "exchange tables (mag, jij_*) are required"; return 1; }

    // ---- merge J, B, D lists per site ------------------------------------
    std::vector<int32_t> cnt(N, 0);
    std::vector<Entry> merged;
    std::vector<int64_t> start(N + 1, 0);
    {
        std::vector<Entry> tmp;
        merged.reserve((size_t)N * (in.j_maxnb + 1));
        out.has_b = in.b_nn != nullptr;
        out.has_d = in.d_nn != nullptr;
        for (int i = 0; i < N; ++i) {
            tmp.clear();
            auto add = [&](int32_t j1, int term, const double *v) -> bool {
                if (j1 < 1 || j1 > N) return false;
                const int32_t j = j1 - 1;
                Entry *e = nullptr;
                for (auto &x : tmp)
                    if (x.j == j) { e = &x; break; }
                if (!e) { tmp.push_back(Entry{j, 0.0, 0.0, {0.0, 0.0, 0.0}}); e = &tmp.back(); }
                if (term == 0) e->J += v[0];
                else if (term == 1) e->B += v[0];
                else { e->D[0] += v[0]; e->D[1] += v[1]; e->D[2] += v[2]; }
                return true;
            };
            const int nj = in.j_nn[i];
            if (nj < 0 || nj > in.j_maxnb) { err = "jij_num_nbors_matrix out of range"; return 1; }
            for (int k = 0; k < nj; ++k) {
                const size_t e = (size_t)k * N + i;
                if (!add(in.j_nbors[e], 0, &in.j_val[e])) { err = "jij_nbors_matrix index out of range"; return 1; }
            }
            if (out.has_b) {
                const int nb = in.b_nn[i];
                if (nb < 0 || nb > in.b_maxnb) { err = "bij_num_nbors_matrix out of range"; return 1; }
                for (int k = 0; k < nb; ++k) {
                    const size_t e = (size_t)k * N + i;
                    if (!add(in.b_nbors[e], 1, &in.b_val[e])) { err = "bij_nbors_matrix index out of range"; return 1; }
                }
            }
            if (out.has_d) {
                const int nd = in.d_nn[i];
                if (nd < 0 || nd > in.d_maxnb) { err = "dij_num_nbors_matrix out of range"; return 1; }
                for (int k = 0; k < nd; ++k) {
                    const size_t e = (size_t)k * N + i;
                    if (!add(in.d_nbors[e], 2, &in.d_val[3 * e])) { err = "dij_nbors_matrix index out of range"; return 1; }
                }
            }
            for (auto &x : tmp)
                if (x.j == i) { err = "a site is bonded to itself (supercell too small for the shells)"; return 1; }
            cnt[i] = (int32_t)tmp.size();
            start[i + 1] = start[i] + (int64_t)tmp.size();
            merged.insert(merged.end(), tmp.begin(), tmp.end());
        }
    }
    int maxnb = 0;
    for (int i = 0; i < N; ++i) maxnb = std::max(maxnb, (int)cnt[i]);
    // device lists are padded to a multiple of kGroup entries
    const int maxnb_pad = ((maxnb + kGroup - 1) / kGroup) * kGroup;
    out.maxnb = maxnb_pad;

    // ---- colouring ---------------------------------------------------------
    std::vector<int> colour(N, -1);
    int C = 0;
    bool done = false;
    const bool all_even = (in.L[0] % 2 == 0) && (in.L[1] % 2 == 0) && (in.L[2] % 2 == 0);
    auto cls_of = [&](int i) {
        const int cell = i / na, at = i % na;
        const int x = cell % in.L[0], y = (cell / in.L[0]) % in.L[1], z = cell / (in.L[0] * in.L[1]);
        return at * 8 + (x & 1) * 4 + (y & 1) * 2 + (z & 1);
    };
    if (all_even && 8 * na <= 512) {
        // parity classes (atom, x mod 2, y mod 2, z mod 2): every bond maps to
        // a pair of classes; colour the class graph, then sites by class.
        const int K = 8 * na;
        std::vector<std::vector<char>> adj(K, std::vector<char>(K, 0));
        bool self = false;
        for (int i = 0; i < N && !self; ++i) {
            const int ci = cls_of(i);
            for (int64_t e = start[i]; e < start[i + 1]; ++e) {
                const int cj = cls_of(merged[e].j);
                if (ci == cj) { self = true; break; }
                adj[ci][cj] = adj[cj][ci] = 1;
            }
        }
        if (!self) {
            std::vector<int> col;
            for (int k = 1; k <= K && !done; ++k) {
                long long budget = 2000000;
                if (colour_k(adj, k, col, budget)) {
                    done = true;
                    // compact used colours
                    std::vector<int> remap(K, -1);
                    int used = 0;
                    for (int c = 0; c < K; ++c)
                        if (col[c] >= 0 && remap[col[c]] < 0) remap[col[c]] = used++;
                    for (int i = 0; i < N; ++i) colour[i] = remap[col[cls_of(i)]];
                    C = used;
                    out.class_colour.assign(K, 0);
                    for (int k = 0; k < K; ++k) out.class_colour[k] = remap[col[k]];
                }
            }
        }
    }
    if (!done) {
        // sequential greedy on the site graph (in reference site order)
        std::vector<int> mark;
        for (int i = 0; i < N; ++i) {
            mark.assign(maxnb + 2, 0);
            for (int64_t e = start[i]; e < start[i + 1]; ++e) {
                const int c = colour[merged[e].j];
                if (c >= 0 && c < (int)mark.size()) mark[c] = 1;
            }
            int c = 0;
            while (mark[c]) ++c;
            colour[i] = c;
            C = std::max(C, c + 1);
        }
    }
    // check: no bond inside a colour class
    for (int i = 0; i < N; ++i)
        for (int64_t e = start[i]; e < start[i + 1]; ++e)
            if (colour[merged[e].j] == colour[i]) { err = "colouring check failed"; return 2; }

    // ---- translation invariance (stencil form) -------------------------------
    if (!out.class_colour.empty() && !in.open_boundary) {
        const int L0 = in.L[0], L1 = in.L[1], L2 = in.L[2];
        auto cell_xyz = [&](int i, int &x, int &y, int &z) {
            const int cell = i / na;
            x = cell % L0; y = (cell / L0) % L1; z = cell / (L0 * L1);
        };
        auto wrap = [](int v, int L) { v %= L; return v < 0 ? v + L : v; };
        auto signed_off = [](int d, int L) { d %= L; if (d < 0) d += L; return d > L / 2 ? d - L : d; };
        bool ok = true;
        std::vector<std::vector<StencilEntry>> st(na);
        for (int a = 0; a < na && ok; ++a) {
            const int i0 = a;  // atom a of cell (0,0,0)
            for (int64_t e = start[i0]; e < start[i0 + 1]; ++e) {
                int x, y, z;
                cell_xyz(merged[e].j, x, y, z);
                StencilEntry se;
                se.dx = signed_off(x, L0); se.dy = signed_off(y, L1); se.dz = signed_off(z, L2);
                se.b = merged[e].j % na;
                se.J = (float)merged[e].J; se.B = (float)merged[e].B;
                se.Dx = (float)merged[e].D[0]; se.Dy = (float)merged[e].D[1]; se.Dz = (float)merged[e].D[2];
                st[a].push_back(se);
            }
        }
        // every site must carry exactly its atom's list, with equal couplings
        // (in the same order, or reordered below to that order)
        for (int i = 0; i < N && ok; ++i) {
            const int a = i % na;
            int x, y, z;
            cell_xyz(i, x, y, z);
            const int64_t n_i = start[i + 1] - start[i];
            if (n_i != (int64_t)st[a].size()) { ok = false; break; }
            auto same = [&](const Entry &m, const StencilEntry &se, int j) {
                return m.j == j && (float)m.J == se.J && (float)m.B == se.B && (float)m.D[0] == se.Dx &&
                       (float)m.D[1] == se.Dy && (float)m.D[2] == se.Dz;
            };
            auto target = [&](const StencilEntry &se) {
                return ((wrap(z + se.dz, L2) * L1 + wrap(y + se.dy, L1)) * L0 + wrap(x + se.dx, L0)) * na + se.b;
            };
            // usual case: the list is already in the stencil's order
            bool in_order = true;
            for (int64_t k = 0; k < n_i && in_order; ++k)
                in_order = same(merged[start[i] + k], st[a][k], target(st[a][k]));
            if (in_order) continue;
            std::vector<Entry> want;
            want.reserve(n_i);
            for (const auto &se : st[a]) {
                const int j = target(se);
                bool found = false;
                for (int64_t e = start[i]; e < start[i + 1]; ++e) {
                    if (same(merged[e], se, j)) {
                        want.push_back(merged[e]);
                        found = true;
                        break;
                    }
                }
                if (!found) { ok = false; break; }
            }
            if (ok) std::copy(want.begin(), want.end(), merged.begin() + start[i]);
        }
        if (ok) {
            out.invariant = true;
            out.stencil = std::move(st);
        }
    }

    // ---- colour-major permutation ------------------------------------------
    out.num_colours = C;
    out.colour = colour;
    out.off.assign(C + 1, 0);
    for (int i = 0; i < N; ++i) out.off[colour[i] + 1]++;
    for (int c = 0; c < C; ++c) out.off[c + 1] += out.off[c];
    out.perm.assign(N, 0);
    out.inv.assign(N, 0);
    if (!out.class_colour.empty()) {
        // parity-class colouring: inside a colour, class by class (ascending
        // class index), and inside a class in site order, which is half-cell
        // order (hz, hy, hx); every class then owns a contiguous block
        const int K = 8 * na;
        std::vector<std::vector<int>> members(K);
        for (int i = 0; i < N; ++i) members[cls_of(i)].push_back(i);
        out.class_off.assign(K, 0);
        int p = 0;
        for (int c = 0; c < C; ++c)
            for (int k = 0; k < K; ++k) {
                if (out.class_colour[k] != c) continue;
                out.class_off[k] = p;
                for (int i : members[k]) {
                    out.perm[p] = i;
                    out.inv[i] = p;
                    ++p;
                }
            }
    } else {
        std::vector<int> fill(out.off.begin(), out.off.end() - 1);
        for (int i = 0; i < N; ++i) {
            const int p = fill[colour[i]]++;
            out.perm[p] = i;
            out.inv[i] = p;
        }
    }
    // ---- pack in permuted order (entry k of site p at k*N + p) -------------
    const size_t M = (size_t)maxnb_pad * N;
    out.nnb.assign(N, 0);
    out.nbr.assign(M, 0);
    out.J.assign(M, 0.f);
    if (out.has_b) out.B.assign(M, 0.f);
    if (out.has_d) { out.Dx.assign(M, 0.f); out.Dy.assign(M, 0.f); out.Dz.assign(M, 0.f); }
    out.mag.assign(N, 0.f);
    for (int p = 0; p < N; ++p) {
        const int i = out.perm[p];
        out.nnb[p] = ((cnt[i] + kGroup - 1) / kGroup) * kGroup;
        out.mag[p] = (float)in.mag[i];
        // padding: zero couplings to the site itself
        for (int k = cnt[i]; k < out.nnb[p]; ++k) out.nbr[(size_t)k * N + p] = p;
        int k = 0;
        for (int64_t e = start[i]; e < start[i + 1]; ++e, ++k) {
            const size_t o = (size_t)k * N + p;
            const Entry &x = merged[e];
            out.nbr[o] = out.inv[x.j];
            out.J[o] = (float)x.J;
            if (out.has_b) out.B[o] = (float)x.B;
            if (out.has_d) { out.Dx[o] = (float)x.D[0]; out.Dy[o] = (float)x.D[1]; out.Dz[o] = (float)x.D[2]; }
        }
    }
    return 0;
}

}  // namespace esp
