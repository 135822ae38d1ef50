// Host-side table preparation (esp_tables.cpp).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace esp {

// Neighbour lists on the device are padded to multiples of this.
constexpr int kGroup = 8;

struct PrepInput {
    int N, num_atoms, L[3];
    bool open_boundary;
    const double *mag;
    int j_maxnb; const int32_t *j_nn, *j_nbors; const double *j_val;
    int b_maxnb; const int32_t *b_nn, *b_nbors; const double *b_val;
    int d_maxnb; const int32_t *d_nn, *d_nbors; const double *d_val;
};

// A translation-invariant interaction: every site of atom a has the same
// neighbour list, given as cell offsets and target atoms.
struct StencilEntry {
    int dx, dy, dz, b;
    float J, B, Dx, Dy, Dz;
};

struct PrepOutput {
    int maxnb = 0, num_colours = 0;  // maxnb: padded list length
    bool has_b = false, has_d = false;
    std::vector<int> colour;      // reference site -> colour
    std::vector<int> off;         // colour c owns permuted sites [off[c], off[c+1])
    std::vector<int> perm, inv;   // permuted -> reference site, and back
    std::vector<int32_t> nnb, nbr;
    std::vector<float> J, B, Dx, Dy, Dz, mag;
    // set when the lattice is periodic, coloured by parity classes and
    // translation invariant: stencil[a] lists the neighbours of atom a in the
    // same order as every site's merged list
    bool invariant = false;
    std::vector<std::vector<StencilEntry>> stencil;
    std::vector<int> class_colour;  // parity class (atom*8 + px*4 + py*2 + pz) -> colour
    std::vector<int> class_off;     // first permuted index of each class (class-major order)
};

// Returns 0 on success, 1 for invalid tables, 2 if the colouring check fails.
int prepare_tables(const PrepInput &in, PrepOutput &out, std::string &err);

}  // namespace esp
