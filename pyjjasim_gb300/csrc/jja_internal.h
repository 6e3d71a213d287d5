// Internal declarations shared by the host factorisation (jja_factor.cpp) and the CUDA
// library (jja_gb300.cu). Not part of the public C ABI (see include/jja_gb300.h).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

namespace jja {

struct FactorOptions {
  int nd_leaf = 8;          // nested-dissection leaf size
  int max_supernode = 0;    // cap on supernode width (0 = none)
  int keep_factor = 0;      // keep the plain Cholesky columns (host checks only)
  int relax_zeros = 16;     // amalgamate a child supernode when it adds at most this many zeros ...
  double relax_frac = 0.05; // ... or at most this fraction of the merged block's entries
};

// P K P^T = L L^T, stored per supernode as F_s = [inv(L11); L21 inv(L11)] ((k+m) x k,
// column-major). perm[new] = old, iperm[old] = new. Supernodes are in postorder.
struct Factor {
  int n = 0, ns = 0, n_levels = 0;
  std::vector<int> perm, iperm;
  std::vector<int> sn_col0, sn_k, sn_m, sn_parent, sn_level;
  std::vector<int64_t> sn_rowptr;  // ns+1, into rows
  std::vector<int> rows;           // off-diagonal row indices (new numbering), ascending
  std::vector<int64_t> sn_valptr;  // ns+1, into fcol
  std::vector<double> fcol;        // F_s blocks, column-major
  std::vector<double> lcol;        // optional: Cholesky columns [L11; L21] (same layout)
  double factor_flops = 0.0;
  int64_t nnz_L = 0;
};

Factor* factor_create(int n, const int64_t* colptr, const int32_t* rowind, const double* val,
                      const double* cx, const double* cy, const int32_t* user_perm, const FactorOptions& opt);
void factor_solve_host(const Factor& F, double* b, int nrhs);

}  // namespace jja
