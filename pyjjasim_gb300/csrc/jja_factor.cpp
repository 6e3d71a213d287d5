// Host-side ordering and supernodal Cholesky factorisation of the face-space matrix
//   K = A (L + diag(1/(C/dt^2 + 1/(R dt)))) A^T            (pyjjasim time_evolution.py:504-506)
// The reference factorises K with SuperLU through scipy.sparse.linalg.factorized once per
// compute() and calls the solve every step (time_evolution.py:562-569). Here K (symmetric
// positive definite) is ordered by nested dissection, factorised once in FP64 as
// P K P^T = L L^T with a multifrontal supernodal Cholesky, and each supernode s (columns
// [c0, c0+k), off-diagonal rows R_s, |R_s| = m) is converted to the block
//     F_s = [ inv(L11) ; L21 inv(L11) ]          ((k+m) x k)
// so that the GPU triangular solves become small dense products with no sequential
// dependence inside a supernode:
//     forward : z_s = inv(L11) b_s ,  b[R_s] -= (L21 inv(L11)) b_s
//     backward: x_s = inv(L11)^T z_s - (L21 inv(L11))^T x[R_s]
// Supernodes are grouped into levels of the supernodal elimination tree (leaves = level 0);
// all supernodes of one level are independent.
#include "jja_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

namespace jja {

// ------------------------------------------------------------------------------------------
// ordering
// ------------------------------------------------------------------------------------------
namespace {

struct Graph {  // symmetric adjacency without the diagonal, CSR
  int n = 0;
  std::vector<int64_t> ptr;
  std::vector<int> adj;
};

Graph pattern_graph(int n, const int64_t* colptr, const int32_t* rowind) {
  Graph g;
  g.n = n;
  std::vector<int64_t> cnt(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) {
      int i = rowind[p];
      if (i == j) continue;
      cnt[i + 1]++;
      cnt[j + 1]++;
    }
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> tmp(cnt[n]);
  std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
  for (int j = 0; j < n; ++j)
    for (int64_t p = colptr[j]; p < colptr[j + 1]; ++p) {
      int i = rowind[p];
      if (i == j) continue;
      tmp[pos[i]++] = j;
      tmp[pos[j]++] = i;
    }
  // sort + dedupe each row (the input holds both triangles, so every pair appears twice)
  g.ptr.assign(n + 1, 0);
  g.adj.reserve(tmp.size() / 2 + 1);
  for (int i = 0; i < n; ++i) {
    auto b = tmp.begin() + cnt[i], e = tmp.begin() + cnt[i + 1];
    std::sort(b, e);
    e = std::unique(b, e);
    g.adj.insert(g.adj.end(), b, e);
    g.ptr[i + 1] = (int64_t)g.adj.size();
  }
  return g;
}

// BFS distances from src inside the vertex subset marked with `tag` in `mark`.
int bfs(const Graph& g, const std::vector<int>& verts, const std::vector<int>& mark, int tag, int src,
        std::vector<int>& dist, std::vector<int>& queue) {
  for (int v : verts) dist[v] = -1;
  int head = 0, tail = 0, last = src;
  queue[tail++] = src;
  dist[src] = 0;
  while (head < tail) {
    int v = queue[head++];
    last = v;
    for (int64_t p = g.ptr[v]; p < g.ptr[v + 1]; ++p) {
      int u = g.adj[p];
      if (mark[u] != tag || dist[u] >= 0) continue;
      dist[u] = dist[v] + 1;
      queue[tail++] = u;
    }
  }
  return last;
}

// Nested dissection. Each subdomain is split at the median of its longest coordinate
// extent (face centroids for lattices); the vertex separator is the set of vertices on the
// upper side that touch the lower side. Subdomains, then their separator, are numbered
// bottom-up so separators come last. Disconnected pieces and coordinate ties are handled
// by falling back to BFS-distance coordinates.
void nested_dissection(const Graph& g, const double* cx, const double* cy, int leaf, std::vector<int>& order) {
  const int n = g.n;
  std::vector<double> X(n), Y(n);
  std::vector<int> mark(n, 0), dist(n), queue(n);
  if (cx && cy) {
    for (int i = 0; i < n; ++i) { X[i] = cx[i]; Y[i] = cy[i]; }
  } else {
    // two BFS sweeps from far-apart vertices give a rough planar-like embedding per component
    std::vector<int> all(n);
    std::iota(all.begin(), all.end(), 0);
    std::vector<int> seen(n, 0);
    for (int s = 0; s < n; ++s) {
      if (seen[s]) continue;
      std::vector<int> comp;
      // collect component
      int head = 0;
      comp.push_back(s);
      seen[s] = 1;
      while (head < (int)comp.size()) {
        int v = comp[head++];
        for (int64_t p = g.ptr[v]; p < g.ptr[v + 1]; ++p)
          if (!seen[g.adj[p]]) { seen[g.adj[p]] = 1; comp.push_back(g.adj[p]); }
      }
      for (int v : comp) mark[v] = 1;
      int a = bfs(g, comp, mark, 1, s, dist, queue);
      int b = bfs(g, comp, mark, 1, a, dist, queue);
      for (int v : comp) X[v] = dist[v];
      bfs(g, comp, mark, 1, b, dist, queue);
      for (int v : comp) Y[v] = dist[v];
      for (int v : comp) mark[v] = 0;
    }
  }
  order.clear();
  order.reserve(n);
  struct Task { std::vector<int> verts; bool emit_only; };
  // explicit stack; a task either splits a domain or emits a separator
  std::vector<Task> stack;
  std::vector<int> all(n);
  std::iota(all.begin(), all.end(), 0);
  stack.push_back({std::move(all), false});
  int tagc = 1;
  while (!stack.empty()) {
    Task t = std::move(stack.back());
    stack.pop_back();
    std::vector<int>& V = t.verts;
    if (t.emit_only || (int)V.size() <= leaf) {
      // leaves: keep the coordinate order (rows of faces) which keeps local fill small
      if (!t.emit_only)
        std::sort(V.begin(), V.end(), [&](int a, int b) { return Y[a] != Y[b] ? Y[a] < Y[b] : X[a] < X[b]; });
      order.insert(order.end(), V.begin(), V.end());
      continue;
    }
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
    for (int v : V) {
      xmin = std::min(xmin, X[v]); xmax = std::max(xmax, X[v]);
      ymin = std::min(ymin, Y[v]); ymax = std::max(ymax, Y[v]);
    }
    const bool use_x = (xmax - xmin) >= (ymax - ymin);
    const std::vector<double>& C = use_x ? X : Y;
    std::vector<double> vals(V.size());
    for (size_t i = 0; i < V.size(); ++i) vals[i] = C[V[i]];
    std::nth_element(vals.begin(), vals.begin() + vals.size() / 2, vals.end());
    double med = vals[vals.size() / 2];
    ++tagc;
    const int tag_lo = tagc;
    ++tagc;
    const int tag_hi = tagc;
    std::vector<int> lo, hi;
    for (int v : V) {
      if (C[v] < med) { lo.push_back(v); mark[v] = tag_lo; }
      else { hi.push_back(v); mark[v] = tag_hi; }
    }
    if (lo.empty() || hi.empty()) {  // all coordinates equal: split by position instead
      lo.assign(V.begin(), V.begin() + V.size() / 2);
      hi.assign(V.begin() + V.size() / 2, V.end());
      for (int v : lo) mark[v] = tag_lo;
      for (int v : hi) mark[v] = tag_hi;
    }
    // separator: the smaller of (hi touching lo) and (lo touching hi)
    std::vector<int> sep_hi, rest_hi, sep_lo, rest_lo;
    for (int v : hi) {
      bool touch = false;
      for (int64_t p = g.ptr[v]; p < g.ptr[v + 1] && !touch; ++p) touch = mark[g.adj[p]] == tag_lo;
      (touch ? sep_hi : rest_hi).push_back(v);
    }
    for (int v : lo) {
      bool touch = false;
      for (int64_t p = g.ptr[v]; p < g.ptr[v + 1] && !touch; ++p) touch = mark[g.adj[p]] == tag_hi;
      (touch ? sep_lo : rest_lo).push_back(v);
    }
    std::vector<int> A, B, S;
    if (sep_hi.size() <= sep_lo.size()) { A = lo; B = rest_hi; S = sep_hi; }
    else { A = rest_lo; B = hi; S = sep_lo; }
    if (A.empty() && B.empty()) {  // cannot split further
      order.insert(order.end(), V.begin(), V.end());
      continue;
    }
    std::sort(S.begin(), S.end(), [&](int a, int b) { return C[a] != C[b] ? C[a] < C[b] : (use_x ? Y[a] < Y[b] : X[a] < X[b]); });
    // processing order: A, B, then S  (stack: push in reverse)
    stack.push_back({std::move(S), true});
    if (!B.empty()) stack.push_back({std::move(B), false});
    if (!A.empty()) stack.push_back({std::move(A), false});
  }
}

}  // namespace

// ------------------------------------------------------------------------------------------
// dense kernels (column-major, leading dimension ld)
// ------------------------------------------------------------------------------------------
namespace {

// In-place lower Cholesky of the k x k leading block of a (ld x *) column-major array.
bool dense_cholesky(double* a, int k, int ld) {
  for (int j = 0; j < k; ++j) {
    double* cj = a + (int64_t)j * ld;
    // left-looking column update: a[j:, j] -= a[j:, 0:j] a[j, 0:j]^T
    for (int p = 0; p < j; ++p) {
      const double* cp = a + (int64_t)p * ld;
      const double f = cp[j];
      if (f == 0.0) continue;
      for (int i = j; i < k; ++i) cj[i] -= cp[i] * f;
    }
    double d = cj[j];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    cj[j] = d;
    const double inv = 1.0 / d;
    for (int i = j + 1; i < k; ++i) cj[i] *= inv;
  }
  return true;
}

// B (m x k, rows offset `off` inside the column-major front, ld) := B inv(L11)^T,
// where L11 is the k x k leading lower block of the same front.
void dense_trsm_right_lt(double* front, int k, int m, int ld) {
  if (m == 0) return;
  for (int j = 0; j < k; ++j) {
    double* bj = front + (int64_t)j * ld + k;
    for (int p = 0; p < j; ++p) {
      const double f = front[(int64_t)p * ld + j];
      if (f == 0.0) continue;
      const double* bp = front + (int64_t)p * ld + k;
      for (int i = 0; i < m; ++i) bj[i] -= bp[i] * f;
    }
    const double inv = 1.0 / front[(int64_t)j * ld + j];
    for (int i = 0; i < m; ++i) bj[i] *= inv;
  }
}

// U (m x m lower, column-major, ld m) = F22 - L21 L21^T  where L21 = front rows k.., cols 0..k-1.
void dense_update(const double* front, int k, int m, int ld, double* U) {
  // copy lower part of F22
  for (int c = 0; c < m; ++c) {
    const double* src = front + (int64_t)(k + c) * ld + k;
    double* dst = U + (int64_t)c * m;
    for (int r = c; r < m; ++r) dst[r] = src[r];
  }
  // blocked rank-k update, column by column of U, 4 columns of L21 at a time
  for (int c = 0; c < m; ++c) {
    double* uc = U + (int64_t)c * m;
    int p = 0;
    for (; p + 4 <= k; p += 4) {
      const double* l0 = front + (int64_t)(p + 0) * ld + k;
      const double* l1 = front + (int64_t)(p + 1) * ld + k;
      const double* l2 = front + (int64_t)(p + 2) * ld + k;
      const double* l3 = front + (int64_t)(p + 3) * ld + k;
      const double f0 = l0[c], f1 = l1[c], f2 = l2[c], f3 = l3[c];
      for (int r = c; r < m; ++r) uc[r] -= l0[r] * f0 + l1[r] * f1 + l2[r] * f2 + l3[r] * f3;
    }
    for (; p < k; ++p) {
      const double* l0 = front + (int64_t)p * ld + k;
      const double f0 = l0[c];
      for (int r = c; r < m; ++r) uc[r] -= l0[r] * f0;
    }
  }
}

// inverse of a k x k lower-triangular (column-major, ld) into out (k x k column-major, ld k)
void dense_tri_inverse(const double* l, int k, int ld, double* out) {
  std::fill(out, out + (int64_t)k * k, 0.0);
  for (int j = 0; j < k; ++j) {
    // column j of inv(L): forward substitution of L x = e_j (x[i] = 0 for i < j)
    double* x = out + (int64_t)j * k;
    x[j] = 1.0;
    for (int p = j; p < k; ++p) {
      const double* lp = l + (int64_t)p * ld;
      const double v = x[p] / lp[p];
      x[p] = v;
      if (v == 0.0) continue;
      for (int i = p + 1; i < k; ++i) x[i] -= lp[i] * v;
    }
  }
}

}  // namespace

// ------------------------------------------------------------------------------------------
// symbolic + numeric factorisation
// ------------------------------------------------------------------------------------------
Factor* factor_create(int n, const int64_t* colptr, const int32_t* rowind, const double* val,
                      const double* cx, const double* cy, const int32_t* user_perm, const FactorOptions& opt) {
  auto F = std::make_unique<Factor>();
  F->n = n;
  if (n <= 0) throw std::runtime_error("empty matrix");
  Graph g = pattern_graph(n, colptr, rowind);

  // 1. fill-reducing order (new -> old)
  std::vector<int> order;
  if (user_perm) {
    order.assign(user_perm, user_perm + n);
    std::vector<char> seen(n, 0);
    for (int v : order) {
      if (v < 0 || v >= n || seen[v]) throw std::runtime_error("user permutation is not a permutation");
      seen[v] = 1;
    }
  } else {
    nested_dissection(g, cx, cy, std::max(1, opt.nd_leaf), order);
  }
  std::vector<int> inv(n);
  for (int i = 0; i < n; ++i) inv[order[i]] = i;

  // 2. elimination tree of the permuted matrix (ancestor path compression)
  std::vector<int> parent(n, -1), anc(n, -1);
  for (int j = 0; j < n; ++j) {
    int oj = order[j];
    for (int64_t p = g.ptr[oj]; p < g.ptr[oj + 1]; ++p) {
      int i = inv[g.adj[p]];
      if (i >= j) continue;
      int r = i;
      while (anc[r] != -1 && anc[r] != j) { int t = anc[r]; anc[r] = j; r = t; }
      if (anc[r] == -1) { anc[r] = j; parent[r] = j; }
    }
  }
  // 3. postorder so every subtree is contiguous and children precede parents
  std::vector<int> head(n, -1), next(n, -1), post;
  post.reserve(n);
  for (int j = n - 1; j >= 0; --j)
    if (parent[j] >= 0) { next[j] = head[parent[j]]; head[parent[j]] = j; }
  {
    std::vector<int> st;
    for (int r = 0; r < n; ++r) {
      if (parent[r] != -1) continue;
      st.push_back(r);
      while (!st.empty()) {
        int v = st.back();
        if (head[v] >= 0) { int c = head[v]; head[v] = next[c]; st.push_back(c); }
        else { st.pop_back(); post.push_back(v); }
      }
    }
  }
  std::vector<int> newpos(n);
  for (int i = 0; i < n; ++i) newpos[post[i]] = i;
  F->perm.resize(n);
  F->iperm.resize(n);
  for (int i = 0; i < n; ++i) F->perm[i] = order[post[i]];
  for (int i = 0; i < n; ++i) F->iperm[F->perm[i]] = i;
  {
    std::vector<int> p2(n, -1);
    for (int j = 0; j < n; ++j) p2[newpos[j]] = parent[j] >= 0 ? newpos[parent[j]] : -1;
    parent.swap(p2);
  }
  const std::vector<int>& perm = F->perm;
  const std::vector<int>& ip = F->iperm;

  // 4. column counts (off-diagonal) by row-subtree traversal
  std::vector<int64_t> cc(n, 0);
  {
    std::vector<int> mk(n, -1);
    for (int i = 0; i < n; ++i) {
      mk[i] = i;
      int oi = perm[i];
      for (int64_t p = g.ptr[oi]; p < g.ptr[oi + 1]; ++p) {
        int k = ip[g.adj[p]];
        if (k >= i) continue;
        for (int j = k; mk[j] != i; j = parent[j]) { cc[j]++; mk[j] = i; }
      }
    }
  }
  // 5. fundamental supernodes, then relaxed amalgamation of chains of small supernodes
  std::vector<int> nchild(n, 0);
  for (int j = 0; j < n; ++j) if (parent[j] >= 0) nchild[parent[j]]++;
  std::vector<int> sstart;
  sstart.push_back(0);
  for (int j = 1; j < n; ++j) {
    bool merge = parent[j - 1] == j && cc[j - 1] == cc[j] + 1 && nchild[j] == 1;
    if (merge && opt.max_supernode > 0 && j - sstart.back() >= opt.max_supernode) merge = false;
    if (!merge) sstart.push_back(j);
  }
  sstart.push_back(n);
  // relaxed amalgamation: merge a supernode into its parent when its columns directly
  // precede the parent's and the merge adds few explicit zeros. A child's structure is
  // contained in the parent's columns plus the parent's structure, so the merged block
  // has the parent's off-diagonal rows; the child's columns gain k_c (k_p + m_p - m_c)
  // zero entries. Chains of single-column supernodes (a separator face touching one more
  // ancestor face than its neighbours) collapse, which shortens the level schedule.
  if (opt.relax_zeros > 0 || opt.relax_frac > 0.0) {
    const int nf0 = (int)sstart.size() - 1;
    std::vector<int> c2s(n);
    for (int s = 0; s < nf0; ++s)
      for (int j = sstart[s]; j < sstart[s + 1]; ++j) c2s[j] = s;
    std::vector<int> a(nf0), b(nf0), par(nf0, -1), alive(nf0, 1), rep(nf0);
    std::vector<int64_t> msz(nf0);
    for (int s = 0; s < nf0; ++s) {
      a[s] = sstart[s];
      b[s] = sstart[s + 1];
      msz[s] = cc[b[s] - 1];
      rep[s] = s;
      if (parent[b[s] - 1] >= 0) par[s] = c2s[parent[b[s] - 1]];
    }
    auto find = [&](int x) {
      while (rep[x] != x) { rep[x] = rep[rep[x]]; x = rep[x]; }
      return x;
    };
    for (int s = 0; s < nf0; ++s) {  // postorder: children before parents
      if (par[s] < 0) continue;
      const int p = find(par[s]);
      if (b[s] != a[p]) continue;
      const int64_t kc = b[s] - a[s], kp = b[p] - a[p], mp = msz[p], mc = msz[s];
      const int64_t extra = kc * (kp + mp - mc);
      const int64_t km = kc + kp;
      const double merged = (double)km * (km + 1) / 2.0 + (double)km * mp;
      if (opt.max_supernode > 0 && km > opt.max_supernode) continue;
      if (extra > opt.relax_zeros && extra > opt.relax_frac * merged) continue;
      a[p] = a[s];
      alive[s] = 0;
      rep[s] = p;
    }
    std::vector<int> ns2;
    for (int s = 0; s < nf0; ++s)
      if (alive[s]) ns2.push_back(a[s]);
    ns2.push_back(n);
    sstart.swap(ns2);
  }
  const int ns = (int)sstart.size() - 1;
  std::vector<int> col2sn(n);
  for (int s = 0; s < ns; ++s)
    for (int j = sstart[s]; j < sstart[s + 1]; ++j) col2sn[j] = s;
  std::vector<int> snpar(ns, -1);
  for (int s = 0; s < ns; ++s) {
    int last = sstart[s + 1] - 1;
    if (parent[last] >= 0) snpar[s] = col2sn[parent[last]];
  }

  // 6. supernodal row structures (children before parents in postorder)
  std::vector<std::vector<int>> children(ns);
  for (int s = 0; s < ns; ++s) if (snpar[s] >= 0) children[snpar[s]].push_back(s);
  F->sn_col0.resize(ns);
  F->sn_k.resize(ns);
  F->sn_m.resize(ns);
  F->sn_parent = snpar;
  F->sn_rowptr.assign(ns + 1, 0);
  std::vector<std::vector<int>> rows(ns);
  {
    std::vector<int> mk(n, -1);
    for (int s = 0; s < ns; ++s) {
      const int c0 = sstart[s], c1 = sstart[s + 1];
      std::vector<int>& R = rows[s];
      for (int j = c0; j < c1; ++j) {
        int oj = perm[j];
        for (int64_t p = g.ptr[oj]; p < g.ptr[oj + 1]; ++p) {
          int i = ip[g.adj[p]];
          if (i >= c1 && mk[i] != s) { mk[i] = s; R.push_back(i); }
        }
      }
      for (int c : children[s])
        for (int i : rows[c])
          if (i >= c1 && mk[i] != s) { mk[i] = s; R.push_back(i); }
      std::sort(R.begin(), R.end());
      F->sn_col0[s] = c0;
      F->sn_k[s] = c1 - c0;
      F->sn_m[s] = (int)R.size();
    }
  }
  for (int s = 0; s < ns; ++s) F->sn_rowptr[s + 1] = F->sn_rowptr[s] + F->sn_m[s];
  F->rows.resize(F->sn_rowptr[ns]);
  for (int s = 0; s < ns; ++s) std::copy(rows[s].begin(), rows[s].end(), F->rows.begin() + F->sn_rowptr[s]);

  // 7. numeric multifrontal factorisation; store F_s = [inv(L11); L21 inv(L11)] column-major
  F->sn_valptr.assign(ns + 1, 0);
  for (int s = 0; s < ns; ++s)
    F->sn_valptr[s + 1] = F->sn_valptr[s] + (int64_t)(F->sn_k[s] + F->sn_m[s]) * F->sn_k[s];
  F->fcol.assign(F->sn_valptr[ns], 0.0);
  // value lookup of the original matrix by (new) column: entries of column perm[j]
  std::vector<int> relpos(n, -1);
  struct Update { int s; std::vector<double> U; };
  std::vector<Update> stack;
  double flops = 0.0;
  int64_t nnzL = 0;
  std::vector<double> front, inv11;
  for (int s = 0; s < ns; ++s) {
    const int c0 = F->sn_col0[s], k = F->sn_k[s], m = F->sn_m[s], nf = k + m;
    const int* R = F->rows.data() + F->sn_rowptr[s];
    front.assign((int64_t)nf * nf, 0.0);
    for (int i = 0; i < k; ++i) relpos[c0 + i] = i;
    for (int i = 0; i < m; ++i) relpos[R[i]] = k + i;
    // assemble K entries of columns c0..c0+k-1 (lower part, rows >= column)
    for (int jj = 0; jj < k; ++jj) {
      const int j = c0 + jj, oj = perm[j];
      for (int64_t p = colptr[oj]; p < colptr[oj + 1]; ++p) {
        const int i = ip[rowind[p]];
        if (i < j) continue;
        const int r = relpos[i];
        if (r < 0) throw std::runtime_error("internal: structure miss during assembly");
        front[(int64_t)jj * nf + r] += val[p];
      }
    }
    // extend-add children's update matrices (they sit on top of the stack, last child on top)
    const int nch = (int)children[s].size();
    for (int q = 0; q < nch; ++q) {
      Update& up = stack.back();
      const int c = up.s;
      const int mc = F->sn_m[c];
      const int* Rc = F->rows.data() + F->sn_rowptr[c];
      for (int b = 0; b < mc; ++b) {
        const int cb = relpos[Rc[b]];
        double* dst = front.data() + (int64_t)cb * nf;
        const double* src = up.U.data() + (int64_t)b * mc;
        for (int a = b; a < mc; ++a) dst[relpos[Rc[a]]] += src[a];
      }
      stack.pop_back();
    }
    if (!dense_cholesky(front.data(), k, nf))
      throw std::runtime_error("matrix is not positive definite (supernode " + std::to_string(s) + ")");
    dense_trsm_right_lt(front.data(), k, m, nf);
    if (m > 0) {
      Update up{s, std::vector<double>((int64_t)m * m)};
      dense_update(front.data(), k, m, nf, up.U.data());
      stack.push_back(std::move(up));
    }
    flops += (double)k * k * k / 3.0 + (double)m * k * k + (double)m * m * k;
    nnzL += (int64_t)k * (k + 1) / 2 + (int64_t)m * k;
    // F_s: top k x k = inv(L11); bottom m x k = L21 inv(L11)
    inv11.resize((int64_t)k * k);
    dense_tri_inverse(front.data(), k, nf, inv11.data());
    double* Fs = F->fcol.data() + F->sn_valptr[s];
    for (int j = 0; j < k; ++j) {
      double* col = Fs + (int64_t)j * nf;
      for (int i = 0; i < k; ++i) col[i] = inv11[(int64_t)j * k + i];
      for (int i = 0; i < m; ++i) col[k + i] = 0.0;
    }
    // L21 inv(L11): column j = sum_{p >= j} L21[:, p] * inv11[p, j]
    for (int j = 0; j < k; ++j) {
      double* col = Fs + (int64_t)j * nf + k;
      for (int p = j; p < k; ++p) {
        const double f = inv11[(int64_t)j * k + p];
        if (f == 0.0) continue;
        const double* l = front.data() + (int64_t)p * nf + k;
        for (int i = 0; i < m; ++i) col[i] += l[i] * f;
      }
    }
    // keep the plain Cholesky factor too (for host checks)
    if (opt.keep_factor) {
      if (F->lcol.empty()) F->lcol.assign(F->sn_valptr[ns], 0.0);
      double* Ls = F->lcol.data() + F->sn_valptr[s];
      for (int j = 0; j < k; ++j)
        for (int i = 0; i < nf; ++i) Ls[(int64_t)j * nf + i] = (i >= j) ? front[(int64_t)j * nf + i] : 0.0;
    }
    for (int i = 0; i < k; ++i) relpos[c0 + i] = -1;
    for (int i = 0; i < m; ++i) relpos[R[i]] = -1;
  }
  F->factor_flops = flops;
  F->nnz_L = nnzL;

  // 8. levels of the supernodal elimination tree
  F->sn_level.assign(ns, 0);
  int maxlev = 0;
  for (int s = 0; s < ns; ++s) {
    if (snpar[s] >= 0) F->sn_level[snpar[s]] = std::max(F->sn_level[snpar[s]], F->sn_level[s] + 1);
    maxlev = std::max(maxlev, F->sn_level[s]);
  }
  F->n_levels = maxlev + 1;
  F->ns = ns;
  return F.release();
}

// Host triangular solves with the F_s blocks (diagnostic: used by tests to check the factor;
// the time-stepping path solves on the GPU only). b is (n x nrhs) row-major, original order.
void factor_solve_host(const Factor& F, double* b, int nrhs) {
  const int n = F.n;
  std::vector<double> y((int64_t)n * nrhs), z((int64_t)n * nrhs, 0.0), x((int64_t)n * nrhs, 0.0);
  for (int i = 0; i < n; ++i)
    for (int w = 0; w < nrhs; ++w) y[(int64_t)i * nrhs + w] = b[(int64_t)F.perm[i] * nrhs + w];
  std::vector<double> bs;
  for (int s = 0; s < F.ns; ++s) {  // forward, children first
    const int c0 = F.sn_col0[s], k = F.sn_k[s], m = F.sn_m[s], nf = k + m;
    const double* Fs = F.fcol.data() + F.sn_valptr[s];
    const int* R = F.rows.data() + F.sn_rowptr[s];
    bs.assign(y.begin() + (int64_t)c0 * nrhs, y.begin() + (int64_t)(c0 + k) * nrhs);
    for (int r = 0; r < nf; ++r)
      for (int w = 0; w < nrhs; ++w) {
        double acc = 0.0;
        for (int j = 0; j < k; ++j) acc += Fs[(int64_t)j * nf + r] * bs[(int64_t)j * nrhs + w];
        if (r < k) z[(int64_t)(c0 + r) * nrhs + w] = acc;
        else y[(int64_t)R[r - k] * nrhs + w] -= acc;
      }
  }
  for (int s = F.ns - 1; s >= 0; --s) {  // backward, parents first
    const int c0 = F.sn_col0[s], k = F.sn_k[s], m = F.sn_m[s], nf = k + m;
    const double* Fs = F.fcol.data() + F.sn_valptr[s];
    const int* R = F.rows.data() + F.sn_rowptr[s];
    for (int i = 0; i < k; ++i)
      for (int w = 0; w < nrhs; ++w) {
        double acc = 0.0;
        const double* col = Fs + (int64_t)i * nf;
        for (int r = i; r < k; ++r) acc += col[r] * z[(int64_t)(c0 + r) * nrhs + w];
        for (int r = 0; r < m; ++r) acc -= col[k + r] * x[(int64_t)R[r] * nrhs + w];
        x[(int64_t)(c0 + i) * nrhs + w] = acc;
      }
  }
  for (int i = 0; i < n; ++i)
    for (int w = 0; w < nrhs; ++w) b[(int64_t)F.perm[i] * nrhs + w] = x[(int64_t)i * nrhs + w];
}

}  // namespace jja
