// Static (stationary) problems on the GPU: the reference's Newton iteration static_compute
// (pyjjasim static_problem.py:1400-1515) and its London approximation (:1378-1395), for W
// problems on one circuit at once. Included by jja_gb300.cu (one translation unit: it reuses the
// sweep item functions, the face tables and the integer-pipe sine of the time-stepping path).
//
// Every Newton iteration solves A S A^T j = r with S = L + diag(1/q), q = Ic cos(theta) per
// problem: a new matrix per iteration and problem, symmetric but indefinite where cos(theta) < 0.
// Its sparsity pattern is fixed, so the host's symbolic supernodal structure (ordering,
// supernodes, row lists, elimination-tree levels) is computed once and every iteration refactors
// numerically on the device, level by level (leaves first), one thread block per (supernode,
// problem): assemble the front from A L A^T and the junction terms 1/q_j, extend-add the children's
// update matrices, eliminate the supernode's k columns (right-looking LDL^T, no pivoting), keep
// the Schur complement for the parent, and write the solve blocks
//     F_s = [ |D_s|^(-1/2) inv(L11) ; L21 inv(L11) ]      (L unit lower, D the pivots)
// i.e. the blocks of P K P^T = Lt S Lt^T with Lt = L |D|^(1/2) and S = sign(D). The triangular
// sweeps of the time-stepping path then solve with those blocks (forward, z *= S, backward),
// each problem with its own factor values.
//
// Layout: the Newton state is problem-major, (W, Nj) / (W, Nf) with the factor's face order for
// face vectors; factor values, update matrices and fronts are held per problem.

namespace {

constexpr int kStaticSmemFront = 158;   // fronts of at most this many rows are factorised in shared memory
constexpr double kPivotTiny = 1e-300;

struct StaticDev {
  FactorDev F;                 // symbolic structure; fcol / frow point at problem 0's values
  int64_t nF;                  // factor values per problem
  int Nj, Nf, W;
  // front assembly: per supernode, the front positions it sets (CSR over supernodes), each with a
  // constant (A L A^T) and a list of junction terms (junction << 1) | (A_pj A_qj is -1)
  const int64_t* pos_ptr;
  const int32_t* pos_idx;
  const double* pos_const;
  const int64_t* pos_cptr;
  const int32_t* contrib;
  const int32_t* child_ptr;    // children of each supernode (CSR)
  const int32_t* child_list;
  const int32_t* relind;       // per off-diagonal row of a supernode (aligned with F.rows): its index in the parent's front
  const int64_t* upd_off;      // update matrix of supernode s at upd + w upd_total + upd_off[s] (m_s x m_s lower)
  int64_t upd_total;
  double* upd;
  double* fcol;                // W x nF
  double* frow;
  double* sign;                // W x Nf: sign of each pivot (factor face order)
  int* err;                    // [w]: a pivot of problem w was zero or not finite
};

// One (supernode, problem) front: assembly, extend-add, partial LDL^T, update matrix, F_s.
// `gfront` (non-null): the front lives in global memory at gfront + w gl_total + gl_off[s],
// else in dynamic shared memory (nf x nf doubles, column-major; the strictly upper part of the
// leading k x k block holds inv(L11) once the columns are eliminated).
__global__ void __launch_bounds__(256) k_st_front(StaticDev S, const int32_t* __restrict__ sn_list,
                                                  double* __restrict__ gfront, int64_t gl_total,
                                                  const int64_t* __restrict__ gl_off, const double* __restrict__ iq,
                                                  const int* __restrict__ active) {
  extern __shared__ double smem_front[];
  const int s = sn_list[blockIdx.x], w = blockIdx.y;
  if (active && !active[w]) return;
  const int k = S.F.k[s], m = S.F.m[s], nf = k + m, c0 = S.F.col0[s];
  double* Fr = gfront ? gfront + (int64_t)w * gl_total + gl_off[s] : smem_front;
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  const int64_t nf2 = (int64_t)nf * nf;
  for (int64_t i = tid; i < nf2; i += nt) Fr[i] = 0.0;
  __syncthreads();
  // entries of K = A (L + diag(1/q)) A^T in the supernode's columns (lower part)
  const double* iqw = iq + (int64_t)w * S.Nj;
  for (int64_t e = S.pos_ptr[s] + tid; e < S.pos_ptr[s + 1]; e += nt) {
    double v = S.pos_const[e];
    for (int64_t c = S.pos_cptr[e]; c < S.pos_cptr[e + 1]; ++c) {
      const int code = S.contrib[c];
      const double x = iqw[code >> 1];
      v += (code & 1) ? -x : x;
    }
    Fr[S.pos_idx[e]] = v;
  }
  __syncthreads();
  // extend-add the children's update matrices (one child at a time: two children may add to
  // the same entry; within a child every (a, b) maps to a distinct entry)
  for (int q = S.child_ptr[s]; q < S.child_ptr[s + 1]; ++q) {
    const int c = S.child_list[q];
    const int mc = S.F.m[c];
    const int32_t* rel = S.relind + S.F.rowptr[c];
    const double* U = S.upd + (int64_t)w * S.upd_total + S.upd_off[c];
    for (int b = warp; b < mc; b += nw) {
      const int64_t cb = (int64_t)rel[b] * nf;
      for (int a = b + lane; a < mc; a += 32) Fr[cb + rel[a]] += U[(int64_t)b * mc + a];
    }
    __syncthreads();
  }
  // right-looking LDL^T of the leading k columns; the trailing block becomes the Schur complement
  bool bad = false;
  for (int j = 0; j < k; ++j) {
    const double d = Fr[(int64_t)j * nf + j];
    bad |= !(fabs(d) > kPivotTiny) || non_finite(d);
    const double inv = 1.0 / d;
    const double* colj = Fr + (int64_t)j * nf;
    for (int c = j + 1 + warp; c < nf; c += nw) {
      const double fc = colj[c] * inv;
      double* colc = Fr + (int64_t)c * nf;
      for (int r = c + lane; r < nf; r += 32) colc[r] -= colj[r] * fc;
    }
    __syncthreads();
    for (int r = j + 1 + tid; r < nf; r += nt) Fr[(int64_t)j * nf + r] *= inv;
    __syncthreads();
  }
  if (bad && tid == 0) S.err[w] = 1;
  // Schur complement -> the parent's update matrix
  if (m > 0) {
    double* U = S.upd + (int64_t)w * S.upd_total + S.upd_off[s];
    for (int b = warp; b < m; b += nw)
      for (int a = b + lane; a < m; a += 32) U[(int64_t)b * m + a] = Fr[(int64_t)(k + b) * nf + k + a];
  }
  // X = inv(L11), L11 unit lower: X[i][j] = -(L[i][j] + sum_{j<p<i} L[i][p] X[p][j]), stored at Fr[i nf + j]
  for (int i = 1; i < k; ++i) {
    for (int j = tid; j < i; j += nt) {
      double acc = Fr[(int64_t)j * nf + i];
      for (int p = j + 1; p < i; ++p) acc = fma(Fr[(int64_t)p * nf + i], Fr[(int64_t)p * nf + j], acc);
      Fr[(int64_t)i * nf + j] = -acc;
    }
    __syncthreads();
  }
  // F_s: rows r < k: |d_r|^(-1/2) X[r][j]; rows k + a: (L21 X)[a][j]; column-major and row-major copies
  double* Fc = S.fcol + (int64_t)w * S.nF + S.F.valptr[s];
  double* Fw = S.frow + (int64_t)w * S.nF + S.F.valptr[s];
  for (int64_t e = tid; e < (int64_t)nf * k; e += nt) {
    const int j = (int)(e / nf), r = (int)(e - (int64_t)j * nf);
    double v;
    if (r < k) {
      const double x = r < j ? 0.0 : (r == j ? 1.0 : Fr[(int64_t)r * nf + j]);
      v = x / sqrt(fabs(Fr[(int64_t)r * nf + r]));
    } else {
      v = Fr[(int64_t)j * nf + r];
      for (int p = j + 1; p < k; ++p) v = fma(Fr[(int64_t)p * nf + r], Fr[(int64_t)p * nf + j], v);
    }
    Fc[e] = v;
    Fw[(int64_t)r * k + j] = v;
  }
  for (int r = tid; r < k; r += nt) S.sign[(int64_t)w * S.Nf + c0 + r] = Fr[(int64_t)r * nf + r] < 0.0 ? -1.0 : 1.0;
}

// the level sweeps of the time-stepping path, one problem per blockIdx.y with its own factor
// values and (problem-major) face vectors; W = 1 work items
template <int kRowsPerLane>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_st_fwd(FactorDev F, int64_t fstride,
                                                                const int4* __restrict__ items, int n_items,
                                                                double* __restrict__ b, double* __restrict__ z,
                                                                int64_t vstride) {
  const int it = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (it >= n_items) return;
  const int w = blockIdx.y;
  FactorDev Fw = F;
  Fw.fcol += (int64_t)w * fstride;
  Fw.frow += (int64_t)w * fstride;
  fwd_item<kRowsPerLane, false>(Fw, unpack_item(items[it]), threadIdx.x & 31, 1, 1, b + (int64_t)w * vstride,
                                z + (int64_t)w * vstride);
}

template <int kRowsPerLane>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_st_bwd(FactorDev F, int64_t fstride,
                                                                const int4* __restrict__ items, int n_items,
                                                                const double* __restrict__ z, double* __restrict__ x,
                                                                int64_t vstride) {
  const int it = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (it >= n_items) return;
  const int w = blockIdx.y;
  FactorDev Fw = F;
  Fw.fcol += (int64_t)w * fstride;
  Fw.frow += (int64_t)w * fstride;
  bwd_item<kRowsPerLane, false>(Fw, unpack_item(items[it]), threadIdx.x & 31, 1, 1, z + (int64_t)w * vstride,
                                x + (int64_t)w * vstride);
}

// zero the rows partial items accumulate into, for every problem (problem-major vectors)
__global__ void k_st_zero_rows(double* __restrict__ v, const int32_t* __restrict__ rows, int n_rows, int W,
                               int64_t vstride) {
  const int64_t n = (int64_t)n_rows * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = e / n_rows, i = e - w * n_rows;
    v[w * vstride + __ldg(rows + i)] = 0.0;
  }
}

// z *= sign (the pivots' signs between the sweeps)
__global__ void k_st_sign(double* __restrict__ z, const double* __restrict__ sign, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    z[e] *= sign[e];
}

// Newton step setup per (problem, junction) (static_problem.py:1487-1491):
//   q = Ic cos(theta) with |q| < qmin set to qmin (= 0.1 tol), iq = 1/q,
//   y = (I - Is) / q, u = theta - y - L Is.
// London mode (q_from_ic): iq = 1/Ic (0 where |Ic| <= 1e-12), u = iq Is + L Is (static_problem.py:1384-1389).
__global__ void k_st_prep(int Nj, int W, const double* __restrict__ theta, const double* __restrict__ I,
                          const double* __restrict__ Is, const double* __restrict__ LIs, const double* __restrict__ Ic,
                          double qmin, int q_from_ic, const longlong2* __restrict__ tab, double* __restrict__ iq,
                          double* __restrict__ y, double* __restrict__ u, const int* __restrict__ active) {
  const int64_t n = (int64_t)Nj * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = e / Nj, j = e - w * Nj;
    if (active && !active[w]) continue;
    const double ic = __ldg(Ic + j), lis = LIs ? LIs[e] : 0.0;
    if (q_from_ic) {
      const double v = fabs(ic) > 1e-12 ? 1.0 / ic : 0.0;
      iq[e] = v;
      u[e] = v * Is[e] + lis;
      continue;
    }
    double sn, cs;
    fast_sincos(theta[e], tab, sn, cs);
    double q = ic * cs;
    if (fabs(q) < qmin) q = qmin;
    const double yy = (I[e] - Is[e]) / q;
    iq[e] = 1.0 / q;
    y[e] = yy;
    u[e] = theta[e] - yy - lis;
  }
}

// b(w, p) = sgn sum_j A_pj u(w, j) + 2 pi c (f - n)(w, orig(p)) in the factor's face order:
// Newton (sgn = 1, c = 1, n = 0: A (theta - y - L Is) + 2 pi f) and London (sgn = -1, c = -1:
// 2 pi (n - f) - A (iIc + L) Is)
__global__ void k_st_rhs(int Nf, int W, Tables t, const double* __restrict__ u, const double* __restrict__ f,
                         const int32_t* __restrict__ nv, double sgn, int Nj, double* __restrict__ b) {
  const int64_t n = (int64_t)Nf * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = e / Nf, p = e - w * Nf;
    double acc = 0.0;
    const double* uw = u + w * Nj;
    for (int64_t i = __ldg(t.fj_ptr + p); i < __ldg(t.fj_ptr + p + 1); ++i) {
      const int code = __ldg(t.fj_col + i);
      acc += signed_by(uw[code >> 1], code & 1);
    }
    const int64_t o = w * Nf + __ldg(t.face_orig + p);
    const double fo = f ? f[o] : 0.0, no = nv ? (double)nv[o] : 0.0;
    b[e] = sgn * (acc + kTwoPi * (fo - no));
  }
}

// per-problem flag: the face solution holds a NaN or inf (static_problem.py:1493)
__global__ void k_st_nonfinite(const double* __restrict__ x, int Nf, int W, int* __restrict__ flag) {
  const int64_t n = (int64_t)Nf * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    if (non_finite(x[e])) flag[e / Nf] = 1;
}

// theta update (static_problem.py:1493-1497) and I = Ic sin(theta); London mode writes
// theta = iIc (A^T x + Is) instead
__global__ void k_st_update(int Nj, int Nf, int W, Tables t, const double* __restrict__ x,
                            const double* __restrict__ iq, const double* __restrict__ y, const double* __restrict__ Is,
                            const double* __restrict__ Ic, const int* __restrict__ bad, int london,
                            const longlong2* __restrict__ tab, double* __restrict__ theta, double* __restrict__ I,
                            const int* __restrict__ active) {
  const int64_t n = (int64_t)Nj * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = e / Nj, j = e - w * Nj;
    if (active && !active[w]) continue;
    const int p0 = __ldg(t.jf_face + 2 * j), p1 = __ldg(t.jf_face + 2 * j + 1);
    const double* xw = x + w * (int64_t)Nf;
    double v = p0 >= 0 ? signed_by(xw[p0 >> 1], p0 & 1) : 0.0;
    if (p1 >= 0) v += signed_by(xw[p1 >> 1], p1 & 1);
    double th;
    if (london) th = iq[e] * (v + Is[e]);
    else if (bad[w]) th = theta[e] + 1e10;
    else th = theta[e] - (y[e] + v * iq[e]);
    theta[e] = th;
    I[e] = __ldg(Ic + j) * fast_sin(th, tab);
  }
}

// I = Ic sin(theta) per (problem, junction)
__global__ void k_st_currents(int Nj, int W, const double* __restrict__ theta, const double* __restrict__ Ic,
                              const longlong2* __restrict__ tab, double* __restrict__ I) {
  const int64_t n = (int64_t)Nj * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    I[e] = __ldg(Ic + e % Nj) * fast_sin(theta[e], tab);
}

// problem-major face vectors between the original and the factor's face order:
// gather dst(w, i) = src(w, map[i]), or scatter dst(w, map[i]) = src(w, i)
__global__ void k_st_permute(const double* __restrict__ src, double* __restrict__ dst,
                             const int32_t* __restrict__ map, int n, int W, int gather) {
  const int64_t nW = (int64_t)n * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nW; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = e / n, i = e - w * n;
    const int64_t o = w * n + __ldg(map + i);
    if (gather) dst[e] = src[o];
    else dst[o] = src[e];
  }
}

// per-row CSR product out = B v for problem-major vectors (L I, L Is)
__global__ void k_st_spmv(int rows, int cols, int W, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                          const double* __restrict__ val, const double* __restrict__ v, double* __restrict__ out) {
  const int64_t n = (int64_t)rows * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = e / rows, r = e - w * rows;
    double acc = 0.0;
    for (int64_t q = __ldg(rp + r); q < __ldg(rp + r + 1); ++q) acc = fma(__ldg(val + q), v[w * cols + __ldg(ci + q)], acc);
    out[e] = acc;
  }
}

// block sum of one value per thread into acc[slot] (double atomics; the residuals are norms)
__device__ __forceinline__ void block_add(double v, double* acc) {
  __shared__ double part[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) atomicAdd(acc, v);
  }
  __syncthreads();
}

// residual sums per problem (get_kirchhoff_error / get_winding_error, static_problem.py:1108-1130),
// accumulated in acc[w * 8 + k]: 0 |df + A (theta + L I)|^2, 1 faces where A round(theta/2 pi) != -n,
// 2 |M (I - Is)|^2, 3 |theta|^2, 4 |L I|^2, 5 |I|^2. Grid (blocks, W).
__global__ void __launch_bounds__(256) k_st_res_junction(int Nj, const double* __restrict__ theta,
                                                         const double* __restrict__ I, const double* __restrict__ LI,
                                                         double* __restrict__ acc) {
  const int w = blockIdx.y;
  double a3 = 0.0, a4 = 0.0, a5 = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < Nj; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = (int64_t)w * Nj + j;
    a3 += theta[e] * theta[e];
    a5 += I[e] * I[e];
    if (LI) a4 += LI[e] * LI[e];
  }
  block_add(a3, acc + w * 8 + 3);
  block_add(a4, acc + w * 8 + 4);
  block_add(a5, acc + w * 8 + 5);
}

__global__ void __launch_bounds__(256) k_st_res_face(int Nf, int Nj, Tables t, const double* __restrict__ theta,
                                                     const double* __restrict__ LI, const double* __restrict__ f,
                                                     const int32_t* __restrict__ nv, double* __restrict__ acc) {
  const int w = blockIdx.y;
  double a0 = 0.0, a1 = 0.0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < Nf; p += (int64_t)gridDim.x * blockDim.x) {
    double r = 0.0;
    long long wind = 0;
    for (int64_t i = __ldg(t.fj_ptr + p); i < __ldg(t.fj_ptr + p + 1); ++i) {
      const int code = __ldg(t.fj_col + i);
      const int64_t e = (int64_t)w * Nj + (code >> 1);
      const double th = theta[e];
      const double v = th + (LI ? LI[e] : 0.0);
      r += signed_by(v, code & 1);
      const long long k = (long long)rint(th / kTwoPi);
      wind += (code & 1) ? -k : k;
    }
    const int64_t o = (int64_t)w * Nf + __ldg(t.face_orig + p);
    r += kTwoPi * (f ? f[o] : 0.0);
    a0 += r * r;
    a1 += (wind != -(long long)(nv ? nv[o] : 0)) ? 1.0 : 0.0;
  }
  block_add(a0, acc + w * 8 + 0);
  block_add(a1, acc + w * 8 + 1);
}

__global__ void __launch_bounds__(256) k_st_res_node(int Nn, int Nj, const int64_t* __restrict__ rp,
                                                     const int32_t* __restrict__ ci, const double* __restrict__ val,
                                                     const double* __restrict__ I, const double* __restrict__ Is,
                                                     double* __restrict__ acc) {
  const int w = blockIdx.y;
  double a2 = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < Nn; r += (int64_t)gridDim.x * blockDim.x) {
    double b = 0.0;
    for (int64_t q = __ldg(rp + r); q < __ldg(rp + r + 1); ++q) {
      const int64_t e = (int64_t)w * Nj + __ldg(ci + q);
      b = fma(__ldg(val + q), I[e] - Is[e], b);
    }
    a2 += b * b;
  }
  block_add(a2, acc + w * 8 + 2);
}

}  // namespace

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
struct jja_static {
  int Nj = 0, Nf = 0, Nn = 0, W = 0, ns = 0, n_levels = 0;
  StaticDev S{};
  Tables t{};
  int32_t* perm = nullptr;                  // factor face order -> original face
  std::vector<int64_t> fwd_ptr, bwd_ptr;    // W = 1 work items per level (both sweeps, levels ascending)
  int4* fwd_items = nullptr;
  int4* bwd_items = nullptr;
  int32_t* zrows_f = nullptr;
  int32_t* zrows_b = nullptr;
  int nz_f = 0, nz_b = 0;
  struct FrontLaunch {
    int64_t off;      // into sn_order
    int count;
    int threads;
    size_t smem;      // 0: fronts in global memory
    int64_t gl_total; // doubles per problem of the level's global fronts
  };
  std::vector<FrontLaunch> launches;        // levels ascending
  int32_t* sn_order = nullptr;
  int64_t* gl_off = nullptr;
  double* gfront = nullptr;
  const int64_t* l_rp = nullptr;
  const int32_t* l_ci = nullptr;
  const double* l_val = nullptr;
  const int64_t* m_rp = nullptr;
  const int32_t* m_ci = nullptr;
  const double* m_val = nullptr;
  const double* Ic = nullptr;
  double A_norm = 0.0, M_norm = 0.0;
  // work buffers (problem-major)
  double *I = nullptr, *iq = nullptr, *y = nullptr, *u = nullptr, *LIs = nullptr, *LI = nullptr;
  double *b = nullptr, *z = nullptr, *x = nullptr, *acc = nullptr;
  int *bad = nullptr, *active = nullptr;
  std::vector<void*> allocs;
  int64_t bytes = 0;
  ~jja_static() {
    for (void* p : allocs) cudaFree(p);
  }
  template <class T>
  T* up(const T* h, size_t n) {
    T* d = upload(h, n, bytes);
    allocs.push_back(d);
    return d;
  }
};

namespace {

// device LDL^T of A (L + diag(iq_w)) A^T for every active problem, levels ascending
void st_factor(jja_static* sp, cudaStream_t st, const int* active) {
  for (const auto& L : sp->launches) {
    const dim3 grid((unsigned)L.count, (unsigned)sp->W);
    if (L.smem)
      k_st_front<<<grid, L.threads, L.smem, st>>>(sp->S, sp->sn_order + L.off, nullptr, 0, nullptr, sp->iq, active);
    else
      k_st_front<<<grid, L.threads, 0, st>>>(sp->S, sp->sn_order + L.off, sp->gfront, L.gl_total, sp->gl_off, sp->iq,
                                            active);
    g_launches++;
  }
}

// x = K_w^{-1} b for every problem (factor face order, problem-major; b is overwritten)
void st_solve(jja_static* sp, cudaStream_t st) {
  const int W = sp->W;
  const int64_t nfW = (int64_t)sp->Nf * W;
  if (sp->nz_f) {
    k_st_zero_rows<<<grid_for((int64_t)sp->nz_f * W, 256), 256, 0, st>>>(sp->z, sp->zrows_f, sp->nz_f, W, sp->Nf);
    g_launches++;
  }
  for (int l = 0; l < sp->n_levels; ++l) {
    const int n = (int)(sp->fwd_ptr[l + 1] - sp->fwd_ptr[l]);
    if (!n) continue;
    k_st_fwd<1><<<dim3((unsigned)((n + kWarpsPerBlock - 1) / kWarpsPerBlock), (unsigned)W), kWarpsPerBlock * 32, 0,
                  st>>>(sp->S.F, sp->S.nF, sp->fwd_items + sp->fwd_ptr[l], n, sp->b, sp->z, sp->Nf);
    g_launches++;
  }
  k_st_sign<<<grid_for(nfW, 256), 256, 0, st>>>(sp->z, sp->S.sign, nfW);
  g_launches++;
  if (sp->nz_b) {
    k_st_zero_rows<<<grid_for((int64_t)sp->nz_b * W, 256), 256, 0, st>>>(sp->x, sp->zrows_b, sp->nz_b, W, sp->Nf);
    g_launches++;
  }
  for (int l = sp->n_levels - 1; l >= 0; --l) {
    const int n = (int)(sp->bwd_ptr[l + 1] - sp->bwd_ptr[l]);
    if (!n) continue;
    k_st_bwd<1><<<dim3((unsigned)((n + kWarpsPerBlock - 1) / kWarpsPerBlock), (unsigned)W), kWarpsPerBlock * 32, 0,
                  st>>>(sp->S.F, sp->S.nF, sp->bwd_items + sp->bwd_ptr[l], n, sp->z, sp->x, sp->Nf);
    g_launches++;
  }
}

// per-problem residual sums (acc, host copy h_acc: W x 8) of theta / I
void st_residuals(jja_static* sp, const double* theta, const double* Is, const double* f, const int32_t* nv,
                  std::vector<double>& h_acc, cudaStream_t st) {
  const int W = sp->W;
  JJA_CUDA(cudaMemsetAsync(sp->acc, 0, (size_t)W * 8 * sizeof(double), st));
  if (sp->l_rp) {
    k_st_spmv<<<grid_for((int64_t)sp->Nj * W, 256), 256, 0, st>>>(sp->Nj, sp->Nj, W, sp->l_rp, sp->l_ci, sp->l_val,
                                                                  sp->I, sp->LI);
    g_launches++;
  }
  const double* LI = sp->l_rp ? sp->LI : nullptr;
  auto blocks = [](int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 64)); };
  k_st_res_junction<<<dim3(blocks(sp->Nj), (unsigned)W), 256, 0, st>>>(sp->Nj, theta, sp->I, LI, sp->acc);
  k_st_res_face<<<dim3(blocks(sp->Nf), (unsigned)W), 256, 0, st>>>(sp->Nf, sp->Nj, sp->t, theta, LI, f, nv, sp->acc);
  k_st_res_node<<<dim3(blocks(sp->Nn), (unsigned)W), 256, 0, st>>>(sp->Nn, sp->Nj, sp->m_rp, sp->m_ci, sp->m_val,
                                                                   sp->I, Is, sp->acc);
  g_launches += 3;
  h_acc.resize((size_t)W * 8);
  JJA_CUDA(cudaMemcpyAsync(h_acc.data(), sp->acc, (size_t)W * 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
  JJA_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

extern "C" {

int jja_static_create(const jja_static_desc* d, const jja_factor* fac, jja_static** out) {
  return guarded([&] {
    if (!d || !fac || !out) throw Error(JJA_ERR_ARG, "jja_static_create: null argument");
    const jja::Factor& F = *fac->f;
    if (d->Nf != F.n) throw Error(JJA_ERR_ARG, "jja_static_create: factor order != Nf");
    if (d->W <= 0 || d->Nj <= 0 || d->Nn <= 0) throw Error(JJA_ERR_ARG, "jja_static_create: W, Nj, Nn must be positive");
    if (!d->a_rowptr || !d->m_rowptr || !d->Ic) throw Error(JJA_ERR_ARG, "jja_static_create: missing A, M or Ic");
    std::unique_ptr<jja_static> sp(new jja_static);
    const int Nj = d->Nj, Nf = d->Nf, W = d->W, ns = F.ns;
    sp->Nj = Nj; sp->Nf = Nf; sp->Nn = d->Nn; sp->W = W; sp->ns = ns; sp->n_levels = F.n_levels;
    sp->A_norm = d->A_norm; sp->M_norm = d->M_norm;
    const FaceTables ft = face_tables(Nj, Nf, d->a_rowptr, d->a_col, d->a_val, F.perm);
    set_face_tables(sp->t, ft, [&](auto* h, size_t n) { return sp->up(h, n); });
    {
      const std::vector<longlong2> tab = build_sin_table();
      sp->t.sincos = sp->up(tab.data(), tab.size());
    }
    sp->perm = sp->up(F.perm.data(), F.perm.size());
    // symbolic structure and per-problem factor values
    StaticDev& S = sp->S;
    S.F.col0 = sp->up(F.sn_col0.data(), ns);
    S.F.k = sp->up(F.sn_k.data(), ns);
    S.F.m = sp->up(F.sn_m.data(), ns);
    S.F.rowptr = sp->up(F.sn_rowptr.data(), F.sn_rowptr.size());
    S.F.rows = sp->up(F.rows.data(), F.rows.size());
    S.F.valptr = sp->up(F.sn_valptr.data(), F.sn_valptr.size());
    S.nF = F.sn_valptr[ns];
    S.Nj = Nj; S.Nf = Nf; S.W = W;
    S.fcol = sp->up<double>(nullptr, (size_t)W * S.nF);
    S.frow = sp->up<double>(nullptr, (size_t)W * S.nF);
    S.F.fcol = S.fcol;
    S.F.frow = S.frow;
    S.sign = sp->up<double>(nullptr, (size_t)W * Nf);
    S.err = sp->up<int>(nullptr, (size_t)W);
    // front positions: column jj of supernode s, row index (its own columns first, then R_s)
    std::vector<int> sup_of(Nf, -1);
    for (int s = 0; s < ns; ++s)
      for (int i = 0; i < F.sn_k[s]; ++i) sup_of[F.sn_col0[s] + i] = s;
    auto row_index = [&](int s, int r) -> int {
      const int c0 = F.sn_col0[s], k = F.sn_k[s];
      if (r >= c0 && r < c0 + k) return r - c0;
      const int* R = F.rows.data() + F.sn_rowptr[s];
      const int* e = R + F.sn_m[s];
      const int* it = std::lower_bound(R, e, r);
      if (it == e || *it != r) throw Error(JJA_ERR_INTERNAL, "jja_static_create: entry outside the factor's structure");
      return k + (int)(it - R);
    };
    struct Entry {
      int s;
      int pos;
      int code;      // -1: constant, else (junction << 1) | negative
      double val;
    };
    std::vector<Entry> ent;
    auto add = [&](int r, int c, int code, double val) {   // lower entry (r >= c), factor numbering
      if (r < c) std::swap(r, c);
      const int s = sup_of[c];
      const int nf = F.sn_k[s] + F.sn_m[s];
      ent.push_back({s, (c - F.sn_col0[s]) * nf + row_index(s, r), code, val});
    };
    if (d->kl_colptr) {     // A L A^T, constant across iterations
      for (int oc = 0; oc < Nf; ++oc)
        for (int64_t q = d->kl_colptr[oc]; q < d->kl_colptr[oc + 1]; ++q) {
          const int r = F.iperm[d->kl_rowind[q]], c = F.iperm[oc];
          if (r >= c) add(r, c, -1, d->kl_val[q]);
        }
    }
    for (int j = 0; j < Nj; ++j) {   // A diag(1/q) A^T: each junction couples its (at most two) faces
      const int f0 = ft.jf_face[2 * (size_t)j], f1 = ft.jf_face[2 * (size_t)j + 1];
      if (f0 >= 0) add(f0 >> 1, f0 >> 1, j << 1, 0.0);
      if (f1 >= 0) add(f1 >> 1, f1 >> 1, j << 1, 0.0);
      if (f0 >= 0 && f1 >= 0) add(f0 >> 1, f1 >> 1, (j << 1) | ((f0 ^ f1) & 1), 0.0);
    }
    std::sort(ent.begin(), ent.end(), [](const Entry& a, const Entry& b) {
      return a.s != b.s ? a.s < b.s : (a.pos != b.pos ? a.pos < b.pos : a.code < b.code);
    });
    std::vector<int64_t> pos_ptr(ns + 1, 0), pos_cptr(1, 0);
    std::vector<int32_t> pos_idx, contrib;
    std::vector<double> pos_const;
    for (size_t i = 0; i < ent.size();) {
      size_t e = i;
      double cst = 0.0;
      while (e < ent.size() && ent[e].s == ent[i].s && ent[e].pos == ent[i].pos) {
        if (ent[e].code < 0) cst += ent[e].val;
        else contrib.push_back(ent[e].code);
        ++e;
      }
      pos_idx.push_back(ent[i].pos);
      pos_const.push_back(cst);
      pos_cptr.push_back((int64_t)contrib.size());
      pos_ptr[ent[i].s + 1]++;
      i = e;
    }
    for (int s = 0; s < ns; ++s) pos_ptr[s + 1] += pos_ptr[s];
    S.pos_ptr = sp->up(pos_ptr.data(), pos_ptr.size());
    S.pos_idx = sp->up(pos_idx.data(), pos_idx.size());
    S.pos_const = sp->up(pos_const.data(), pos_const.size());
    S.pos_cptr = sp->up(pos_cptr.data(), pos_cptr.size());
    S.contrib = sp->up(contrib.data(), contrib.size());
    // children, their rows' places in the parent's front, update-matrix offsets
    std::vector<int32_t> child_ptr(ns + 1, 0), child_list, relind(F.rows.size(), 0);
    for (int s = 0; s < ns; ++s)
      if (F.sn_parent[s] >= 0) child_ptr[F.sn_parent[s] + 1]++;
    for (int s = 0; s < ns; ++s) child_ptr[s + 1] += child_ptr[s];
    child_list.resize(child_ptr[ns]);
    {
      std::vector<int32_t> fill(child_ptr.begin(), child_ptr.end() - 1);
      for (int s = 0; s < ns; ++s) {
        const int p = F.sn_parent[s];
        if (p < 0) continue;
        child_list[fill[p]++] = s;
        for (int a = 0; a < F.sn_m[s]; ++a)
          relind[F.sn_rowptr[s] + a] = row_index(p, F.rows[F.sn_rowptr[s] + a]);
      }
    }
    S.child_ptr = sp->up(child_ptr.data(), child_ptr.size());
    S.child_list = sp->up(child_list.data(), child_list.size());
    S.relind = sp->up(relind.data(), relind.size());
    std::vector<int64_t> upd_off(ns + 1, 0);
    for (int s = 0; s < ns; ++s) upd_off[s + 1] = upd_off[s] + (int64_t)F.sn_m[s] * F.sn_m[s];
    S.upd_off = sp->up(upd_off.data(), upd_off.size());
    S.upd_total = upd_off[ns];
    S.upd = sp->up<double>(nullptr, (size_t)std::max<int64_t>(1, W * S.upd_total));
    // factorisation launches: per level, fronts grouped by size (shared-memory classes, then the
    // ones that live in global memory)
    std::vector<std::vector<int>> by_level(F.n_levels);
    for (int s = 0; s < ns; ++s) by_level[F.sn_level[s]].push_back(s);
    const int classes[4] = {32, 64, 128, kStaticSmemFront};
    std::vector<int32_t> order;
    std::vector<int64_t> gl_off(ns, 0);
    int64_t gmax = 0;
    for (int l = 0; l < F.n_levels; ++l) {
      for (int ci = 0; ci <= 4; ++ci) {
        const int lo = ci == 0 ? 0 : (ci <= 3 ? classes[ci - 1] : kStaticSmemFront);
        const int hi = ci <= 3 ? classes[ci] : INT_MAX;
        jja_static::FrontLaunch L{(int64_t)order.size(), 0, 256, 0, 0};
        int nfmax = 0;
        for (int s : by_level[l]) {
          const int nf = F.sn_k[s] + F.sn_m[s];
          if (nf <= lo || nf > hi) continue;
          order.push_back(s);
          nfmax = std::max(nfmax, nf);
          if (ci == 4) {
            gl_off[s] = L.gl_total;
            L.gl_total += (int64_t)nf * nf;
          }
        }
        L.count = (int)(order.size() - L.off);
        if (!L.count) continue;
        if (ci < 4) {
          L.smem = (size_t)nfmax * nfmax * sizeof(double);
          L.threads = nfmax <= 32 ? 64 : (nfmax <= 64 ? 128 : 256);
        }
        gmax = std::max(gmax, L.gl_total);
        sp->launches.push_back(L);
      }
    }
    sp->sn_order = sp->up(order.data(), order.size());
    sp->gl_off = sp->up(gl_off.data(), gl_off.size());
    sp->gfront = sp->up<double>(nullptr, (size_t)std::max<int64_t>(1, gmax * W));
    JJA_CUDA(cudaFuncSetAttribute(k_st_front, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)((size_t)kStaticSmemFront * kStaticSmemFront * sizeof(double))));
    // W = 1 sweep items (no lane packs: every problem has its own factor values)
    jja_solve_tuning tu{};
    tu.pack_rows = -1;
    tu.subtree_rows = -1;   // the static sweeps run level items only
    tu.rows_per_lane = 1;
    const Schedule Sch = build_schedule(F, 1, tu);
    sp->fwd_ptr = Sch.fwd_ptr;
    sp->bwd_ptr = Sch.bwd_ptr;
    sp->fwd_items = sp->up(Sch.fi.data(), Sch.fi.size());
    sp->bwd_items = sp->up(Sch.bi.data(), Sch.bi.size());
    sp->nz_f = (int)Sch.zf.size();
    sp->nz_b = (int)Sch.zb.size();
    sp->zrows_f = sp->up(Sch.zf.data(), Sch.zf.size());
    sp->zrows_b = sp->up(Sch.zb.data(), Sch.zb.size());
    // circuit matrices
    if (d->l_rowptr) {
      const int64_t nnz = d->l_rowptr[Nj];
      sp->l_rp = sp->up(d->l_rowptr, (size_t)Nj + 1);
      sp->l_ci = sp->up(d->l_col, (size_t)nnz);
      sp->l_val = sp->up(d->l_val, (size_t)nnz);
    }
    {
      const int64_t nnz = d->m_rowptr[d->Nn];
      sp->m_rp = sp->up(d->m_rowptr, (size_t)d->Nn + 1);
      sp->m_ci = sp->up(d->m_col, (size_t)nnz);
      sp->m_val = sp->up(d->m_val, (size_t)nnz);
    }
    sp->Ic = sp->up(d->Ic, (size_t)Nj);
    const size_t NjW = (size_t)Nj * W, NfW = (size_t)Nf * W;
    sp->I = sp->up<double>(nullptr, NjW);
    sp->iq = sp->up<double>(nullptr, NjW);
    sp->y = sp->up<double>(nullptr, NjW);
    sp->u = sp->up<double>(nullptr, NjW);
    sp->LIs = sp->up<double>(nullptr, NjW);
    sp->LI = sp->up<double>(nullptr, NjW);
    sp->b = sp->up<double>(nullptr, NfW);
    sp->z = sp->up<double>(nullptr, NfW);
    sp->x = sp->up<double>(nullptr, NfW);
    sp->acc = sp->up<double>(nullptr, (size_t)W * 8);
    sp->bad = sp->up<int>(nullptr, (size_t)W);
    sp->active = sp->up<int>(nullptr, (size_t)W);
    JJA_CUDA(cudaDeviceSynchronize());
    *out = sp.release();
  });
}

void jja_static_destroy(jja_static* sp) { delete sp; }

int64_t jja_static_device_bytes(const jja_static* sp) { return sp ? sp->bytes : 0; }

int jja_static_solve(jja_static* sp, const double* iq, const double* b, double* x, int* pivot_errors, void* stream) {
  return guarded([&] {
    if (!sp || !iq || !b || !x) throw Error(JJA_ERR_ARG, "jja_static_solve: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t NjW = (int64_t)sp->Nj * sp->W;
    JJA_CUDA(cudaMemcpyAsync(sp->iq, iq, NjW * sizeof(double), cudaMemcpyDeviceToDevice, st));
    JJA_CUDA(cudaMemsetAsync(sp->S.err, 0, (size_t)sp->W * sizeof(int), st));
    st_factor(sp, st, nullptr);
    k_st_permute<<<grid_for((int64_t)sp->Nf * sp->W, 256), 256, 0, st>>>(b, sp->b, sp->perm, sp->Nf, sp->W, 1);
    st_solve(sp, st);
    k_st_permute<<<grid_for((int64_t)sp->Nf * sp->W, 256), 256, 0, st>>>(sp->x, x, sp->perm, sp->Nf, sp->W, 0);
    g_launches += 2;
    JJA_CUDA(cudaGetLastError());
    if (pivot_errors) {
      JJA_CUDA(cudaMemcpyAsync(pivot_errors, sp->S.err, (size_t)sp->W * sizeof(int), cudaMemcpyDeviceToHost, st));
      JJA_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int jja_static_london(jja_static* sp, const double* Is, const double* f, const int32_t* n, double* theta,
                      void* stream) {
  return guarded([&] {
    if (!sp || !Is || !f || !n || !theta) throw Error(JJA_ERR_ARG, "jja_static_london: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t NjW = (int64_t)sp->Nj * sp->W, NfW = (int64_t)sp->Nf * sp->W;
    const double* LIs = nullptr;
    if (sp->l_rp) {
      k_st_spmv<<<grid_for(NjW, 256), 256, 0, st>>>(sp->Nj, sp->Nj, sp->W, sp->l_rp, sp->l_ci, sp->l_val, Is, sp->LIs);
      g_launches++;
      LIs = sp->LIs;
    }
    k_st_prep<<<grid_for(NjW, 256), 256, 0, st>>>(sp->Nj, sp->W, nullptr, nullptr, Is, LIs, sp->Ic, 0.0, 1,
                                                  sp->t.sincos, sp->iq, sp->y, sp->u, nullptr);
    JJA_CUDA(cudaMemsetAsync(sp->S.err, 0, (size_t)sp->W * sizeof(int), st));
    st_factor(sp, st, nullptr);
    k_st_rhs<<<grid_for(NfW, 256), 256, 0, st>>>(sp->Nf, sp->W, sp->t, sp->u, f, n, -1.0, sp->Nj, sp->b);
    st_solve(sp, st);
    k_st_update<<<grid_for(NjW, 256), 256, 0, st>>>(sp->Nj, sp->Nf, sp->W, sp->t, sp->x, sp->iq, sp->y, Is, sp->Ic,
                                                    nullptr, 1, sp->t.sincos, theta, sp->I, nullptr);
    g_launches += 3;
    JJA_CUDA(cudaGetLastError());
  });
}

int jja_static_newton(jja_static* sp, const jja_newton_args* a, jja_newton_result* r, void* stream) {
  return guarded([&] {
    if (!sp || !a || !r || !a->theta || !a->Is || !a->f || !a->n)
      throw Error(JJA_ERR_ARG, "jja_static_newton: null argument");
    if (a->maxiter < 0) throw Error(JJA_ERR_ARG, "jja_static_newton: maxiter must be >= 0");
    if (!r->status || !r->iterations || !r->residuals || !r->is_target)
      throw Error(JJA_ERR_ARG, "jja_static_newton: missing result array");
    cudaStream_t st = (cudaStream_t)stream;
    const int W = sp->W, Nj = sp->Nj, Nf = sp->Nf, R = a->maxiter + 1;
    const int64_t NjW = (int64_t)Nj * W, NfW = (int64_t)Nf * W;
    double* theta = a->theta;
    // |Is| and |2 pi f| per problem (the reference computes them once, static_problem.py:1470-1474)
    std::vector<double> h_Is((size_t)NjW), h_f((size_t)NfW), Is_norm(W, 0.0), df_norm(W, 0.0);
    JJA_CUDA(cudaMemcpyAsync(h_Is.data(), a->Is, NjW * sizeof(double), cudaMemcpyDeviceToHost, st));
    JJA_CUDA(cudaMemcpyAsync(h_f.data(), a->f, NfW * sizeof(double), cudaMemcpyDeviceToHost, st));
    JJA_CUDA(cudaStreamSynchronize(st));
    for (int w = 0; w < W; ++w) {
      double s1 = 0.0, s2 = 0.0;
      for (int j = 0; j < Nj; ++j) s1 += h_Is[(size_t)w * Nj + j] * h_Is[(size_t)w * Nj + j];
      for (int p = 0; p < Nf; ++p) {
        const double v = kTwoPi * h_f[(size_t)w * Nf + p];
        s2 += v * v;
      }
      Is_norm[w] = std::sqrt(s1);
      df_norm[w] = std::sqrt(s2);
    }
    const double* LIs = nullptr;
    if (sp->l_rp) {
      k_st_spmv<<<grid_for(NjW, 256), 256, 0, st>>>(Nj, Nj, W, sp->l_rp, sp->l_ci, sp->l_val, a->Is, sp->LIs);
      g_launches++;
      LIs = sp->LIs;
    }
    k_st_currents<<<grid_for(NjW, 256), 256, 0, st>>>(Nj, W, theta, sp->Ic, sp->t.sincos, sp->I);
    g_launches++;
    const double eps = std::numeric_limits<double>::epsilon();
    std::vector<double> h_acc;
    std::vector<std::vector<double>> err(W);
    std::vector<std::vector<int>> tgt(W);
    auto record = [&](const std::vector<int>& which) {
      st_residuals(sp, theta, a->Is, a->f, a->n, h_acc, st);
      for (int w : which) {
        const double* c = h_acc.data() + (size_t)w * 8;
        const double kn = sp->M_norm * (Is_norm[w] + std::sqrt(c[5]));
        const double e1 = std::fabs(kn) < 1e-20 ? eps : std::sqrt(c[2]) / kn;
        const double wn = sp->A_norm * (std::sqrt(c[3] / Nj) + std::sqrt(c[4] / Nj)) + df_norm[w] / std::sqrt((double)Nf);
        const double e2 = std::fabs(wn) < 1e-20 ? eps : std::sqrt(c[0] / Nf) / wn;
        err[w].push_back(std::max(e1, e2));
        tgt[w].push_back(c[1] == 0.0 ? 1 : 0);
      }
    };
    std::vector<int> all(W);
    for (int w = 0; w < W; ++w) all[w] = w;
    record(all);
    std::vector<int> iter(W, 0), done(W, 0), h_active(W, 0);
    std::vector<double> prev(W, std::numeric_limits<double>::infinity());
    const double tol = a->tol;
    while (true) {
      std::vector<int> act;
      for (int w = 0; w < W; ++w) {
        if (done[w]) continue;
        const double e = err[w].back();
        const bool t = tgt[w].back() != 0;
        if (e < tol || (e > 0.5 && iter[w] > 5) || (a->stop_if_not_target_n && t) ||
            (a->stop_as_residual_increases && e > prev[w]) || iter[w] >= a->maxiter)
          done[w] = 1;
        else
          act.push_back(w);
      }
      if (act.empty()) break;
      for (int w = 0; w < W; ++w) h_active[w] = done[w] ? 0 : 1;
      JJA_CUDA(cudaMemcpyAsync(sp->active, h_active.data(), (size_t)W * sizeof(int), cudaMemcpyHostToDevice, st));
      k_st_prep<<<grid_for(NjW, 256), 256, 0, st>>>(Nj, W, theta, sp->I, a->Is, LIs, sp->Ic, 0.1 * tol, 0,
                                                    sp->t.sincos, sp->iq, sp->y, sp->u, sp->active);
      k_st_rhs<<<grid_for(NfW, 256), 256, 0, st>>>(Nf, W, sp->t, sp->u, a->f, nullptr, 1.0, Nj, sp->b);
      g_launches += 2;
      st_factor(sp, st, sp->active);
      st_solve(sp, st);
      JJA_CUDA(cudaMemsetAsync(sp->bad, 0, (size_t)W * sizeof(int), st));
      k_st_nonfinite<<<grid_for(NfW, 256), 256, 0, st>>>(sp->x, Nf, W, sp->bad);
      k_st_update<<<grid_for(NjW, 256), 256, 0, st>>>(Nj, Nf, W, sp->t, sp->x, sp->iq, sp->y, a->Is, sp->Ic, sp->bad,
                                                      0, sp->t.sincos, theta, sp->I, sp->active);
      g_launches += 2;
      record(act);
      for (int w : act) {
        if (iter[w] >= 3) prev[w] = err[w][(size_t)iter[w] - 3];
        iter[w]++;
      }
    }
    // NewtonIterInfo.get_status (static_problem.py:116-123): 0 converged on the target vortex
    // configuration, +1 otherwise, +2 when the iteration count reached maxiter
    for (int w = 0; w < W; ++w) {
      const size_t last = err[w].size() - 1;
      const bool found = err[w][last] < tol && tgt[w][last] != 0;
      r->status[w] = (found ? 0 : 1) + 2 * ((int)err[w].size() >= a->maxiter ? 1 : 0);
      r->iterations[w] = iter[w];
      for (int i = 0; i < R; ++i) {
        r->residuals[(size_t)w * R + i] = i < (int)err[w].size() ? err[w][i] : 0.0;
        r->is_target[(size_t)w * R + i] = i < (int)tgt[w].size() ? tgt[w][i] : 0;
      }
    }
    JJA_CUDA(cudaGetLastError());
  });
}

}  // extern "C"
