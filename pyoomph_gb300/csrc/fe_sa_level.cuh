// One level of the smoothed-aggregation hierarchy of the device saddle-point
// solver, built on the host with threads (fe_sa_level_build).  Included by
// fe_gb300.cu after its extern "C" block; host code only.
//
// From the n x n CSR matrix A and its aggregates agg[i] in [0, n_agg):
//   lam = 1.1 x the largest eigenvalue of D^-1 A (12 power iterations from a
//         fixed start vector; D = diag(A)),
//   P   = P0 - (4/3)/lam D^-1 A P0     (n x n_agg; P0 the 0/1 aggregation),
//   Ac  = P^T A P                      (n_agg x n_agg, through AP = A P).
// Every output row is computed on its own (Gustavson's row-by-row product
// with a dense accumulator per thread), sums in a fixed order and lists its
// columns ascending; the power iteration's norms are summed over fixed
// chunks in chunk order.  So the level does not depend on the number of
// threads.

#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

struct fe_sa_level {
  std::vector<int32_t> prp, pci, arp, aci;
  std::vector<double> pv, av;
  double lam = 0.0;
};

namespace fe_sa {

inline unsigned threads_for(int64_t rows) {
  unsigned t = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  return rows < 8192 ? 1u : t;
}

template <class F> void parallel_ranges(int64_t n, unsigned nt, F &&f) {
  if (nt <= 1) {
    f(int64_t(0), n, 0u);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++) th.emplace_back([&, t]() { f(n * t / nt, n * (t + 1) / nt, t); });
  for (auto &x : th) x.join();
}

// dense accumulator over the columns of one output row: value and row
// stamp side by side, so that a term touches one cache line
struct Row {
  struct Slot {
    double acc;
    int32_t mark;
  };
  std::vector<Slot> s;
  std::vector<int32_t> cols;
  int32_t stamp = 0;
  explicit Row(int64_t ncols) : s((size_t)std::max<int64_t>(ncols, 1), Slot{0.0, -1}) {}
  void start() {
    stamp++;
    cols.clear();
  }
  void add(int32_t c, double v) {
    Slot &x = s[c];
    if (x.mark != stamp) {
      x.mark = stamp;
      x.acc = v;
      cols.push_back(c);
    } else {
      x.acc += v;
    }
  }
  double get(int32_t c) const { return s[c].acc; }
};

// CSR of nrows rows over ncols columns, row i filled by fill(i, row)
template <class Fill>
void build_rows(int64_t nrows, int64_t ncols, Fill &&fill, std::vector<int32_t> &rp, std::vector<int32_t> &ci,
                std::vector<double> &v) {
  const unsigned nt = threads_for(nrows);
  std::vector<std::vector<int32_t>> tc(nt);
  std::vector<std::vector<double>> tv(nt);
  std::vector<int64_t> len((size_t)nrows, 0);
  parallel_ranges(nrows, nt, [&](int64_t lo, int64_t hi, unsigned t) {
    // filled locally and moved out at the end: the threads' vectors in tc/tv
    // share cache lines, so growing them in place would contend
    Row row(ncols);
    std::vector<int32_t> c_loc;
    std::vector<double> v_loc;
    for (int64_t i = lo; i < hi; i++) {
      row.start();
      fill(i, row);
      std::sort(row.cols.begin(), row.cols.end());
      for (int32_t c : row.cols) {
        c_loc.push_back(c);
        v_loc.push_back(row.get(c));
      }
      len[i] = (int64_t)row.cols.size();
    }
    tc[t] = std::move(c_loc);
    tv[t] = std::move(v_loc);
  });
  rp.assign((size_t)nrows + 1, 0);
  int64_t total = 0;
  for (int64_t i = 0; i < nrows; i++) {
    total += len[i];
    rp[i + 1] = (int32_t)total;
  }
  ci.clear();
  v.clear();
  ci.reserve((size_t)total);
  v.reserve((size_t)total);
  for (unsigned t = 0; t < nt; t++) {
    ci.insert(ci.end(), tc[t].begin(), tc[t].end());
    v.insert(v.end(), tv[t].begin(), tv[t].end());
  }
}

// sum of squares over fixed chunks, added in chunk order
inline double norm2(const std::vector<double> &x, unsigned nt) {
  const int64_t n = (int64_t)x.size(), chunk = 4096, nc = (n + chunk - 1) / chunk;
  std::vector<double> part((size_t)std::max<int64_t>(nc, 1), 0.0);
  parallel_ranges(nc, nt, [&](int64_t lo, int64_t hi, unsigned) {
    for (int64_t c = lo; c < hi; c++) {
      double s = 0.0;
      for (int64_t i = c * chunk; i < std::min(n, (c + 1) * chunk); i++) s += x[i] * x[i];
      part[c] = s;
    }
  });
  double s = 0.0;
  for (double p : part) s += p;
  return std::sqrt(s);
}

} // namespace fe_sa

extern "C" {

// Aggregates for the smoothed-aggregation hierarchy: greedy over the rows in
// order (roots with a free strong neighbourhood, then joins to a first-pass
// neighbour, then the leftovers), with the strength of connection
// |a_ij| >= theta sqrt(|a_ii| |a_jj|) between unknowns of the same
// component.  The strength flags are computed once per entry, in parallel;
// the greedy passes stay serial, so the aggregates do not depend on the
// number of threads.
int fe_sa_aggregate(int64_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                    const int32_t *comp, double theta, int32_t *agg, int64_t *n_agg) {
  if (n < 0 || (n > 0 && (!rowptr || !colidx || !vals || !comp || !agg)) || !n_agg)
    return fail(FE_ERR_ARG, "fe_sa_aggregate: null argument");
  const unsigned nt = fe_sa::threads_for(n);
  std::vector<double> diag((size_t)n, 0.0);
  std::vector<int> bad(nt, 0);
  fe_sa::parallel_ranges(n, nt, [&](int64_t lo, int64_t hi, unsigned t) {
    for (int64_t i = lo; i < hi; i++)
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
        if (colidx[k] < 0 || colidx[k] >= n) bad[t] = 1;
        else if (colidx[k] == i) diag[i] = std::fabs(vals[k]);
      }
  });
  for (int b : bad)
    if (b) return fail(FE_ERR_ARG, "fe_sa_aggregate: column out of range");
  std::vector<uint8_t> strong(n > 0 ? (size_t)rowptr[n] : 0);
  fe_sa::parallel_ranges(n, nt, [&](int64_t lo, int64_t hi, unsigned) {
    for (int64_t i = lo; i < hi; i++)
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
        const int32_t j = colidx[k];
        strong[k] = j != i && comp[j] == comp[i] && std::fabs(vals[k]) >= theta * std::sqrt(diag[i] * diag[j]);
      }
  });
  for (int64_t i = 0; i < n; i++) agg[i] = -1;
  int32_t na = 0;
  for (int64_t i = 0; i < n; i++) {   // roots with a free strong neighbourhood
    if (agg[i] >= 0) continue;
    bool free_ = true;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1] && free_; k++)
      if (strong[k] && agg[colidx[k]] >= 0) free_ = false;
    if (!free_) continue;
    agg[i] = na;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (strong[k]) agg[colidx[k]] = na;
    na++;
  }
  std::vector<int32_t> first(agg, agg + n);
  for (int64_t i = 0; i < n; i++) {   // join a neighbouring aggregate (of the first pass)
    if (agg[i] >= 0) continue;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (strong[k] && first[colidx[k]] >= 0) {
        agg[i] = first[colidx[k]];
        break;
      }
  }
  for (int64_t i = 0; i < n; i++) {   // leftovers: new aggregates with their free strong neighbours
    if (agg[i] >= 0) continue;
    agg[i] = na;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (strong[k] && agg[colidx[k]] < 0) agg[colidx[k]] = na;
    na++;
  }
  *n_agg = na;
  return FE_OK;
}

int fe_sa_level_build(int64_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals, const int32_t *agg,
                      int64_t n_agg, fe_sa_level_t **out) {
  if (!out) return fail(FE_ERR_ARG, "fe_sa_level_build: null output");
  *out = nullptr;
  if (n <= 0 || n_agg <= 0 || !rowptr || !colidx || !vals || !agg)
    return fail(FE_ERR_ARG, "fe_sa_level_build: empty or null argument");
  if (rowptr[0] != 0 || rowptr[n] < 0) return fail(FE_ERR_ARG, "fe_sa_level_build: bad row pointers");
  for (int64_t i = 0; i < n; i++)
    if (rowptr[i + 1] < rowptr[i]) return fail(FE_ERR_ARG, "fe_sa_level_build: bad row pointers");
  const unsigned nt = fe_sa::threads_for(n);
  std::vector<double> d((size_t)n, 0.0);
  std::vector<int> bad(nt, 0); // 1 aggregate, 2 column, 3 diagonal
  fe_sa::parallel_ranges(n, nt, [&](int64_t lo, int64_t hi, unsigned t) {
    for (int64_t i = lo; i < hi && !bad[t]; i++) {
      if (agg[i] < 0 || agg[i] >= n_agg) bad[t] = 1;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
        if (colidx[k] < 0 || colidx[k] >= n) bad[t] = 2;
        else if (colidx[k] == i) d[i] += vals[k];
      }
      if (!bad[t] && (!(d[i] != 0.0) || !std::isfinite(d[i]))) bad[t] = 3;
    }
  });
  for (int b : bad) {
    if (b == 1) return fail(FE_ERR_ARG, "fe_sa_level_build: aggregate out of range");
    if (b == 2) return fail(FE_ERR_ARG, "fe_sa_level_build: column out of range");
    if (b == 3) return fail(FE_ERR_ARG, "fe_sa_level_build: zero or non-finite diagonal");
  }
  // lam: power iteration on D^-1 A
  std::vector<double> x((size_t)n), y((size_t)n);
  for (int64_t i = 0; i < n; i++) {
    const double f = (double)i * 0.6180339887498949;
    x[i] = 0.5 + (f - std::floor(f));
  }
  double lam = 1.0;
  // y = D^-1 A x over fixed chunks of rows, each chunk also summing x_i^2
  // and y_i^2 in row order (the sums of norm2, fused into the same pass)
  const int64_t chunk = 4096, nch = (n + chunk - 1) / chunk;
  std::vector<double> px((size_t)nch), py((size_t)nch);
  for (int it = 0; it < 12; it++) {
    fe_sa::parallel_ranges(nch, nt, [&](int64_t clo, int64_t chi, unsigned) {
      for (int64_t c = clo; c < chi; c++) {
        double sx = 0.0, sy = 0.0;
        for (int64_t i = c * chunk; i < std::min(n, (c + 1) * chunk); i++) {
          double s = 0.0;
          for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) s += vals[k] * x[colidx[k]];
          y[i] = s / d[i];
          sx += x[i] * x[i];
          sy += y[i] * y[i];
        }
        px[c] = sx;
        py[c] = sy;
      }
    });
    double sx = 0.0, sy = 0.0;
    for (int64_t c = 0; c < nch; c++) {
      sx += px[c];
      sy += py[c];
    }
    const double nx = std::sqrt(sx), ny = std::sqrt(sy);
    lam = ny / std::max(nx, 1e-300);
    const double sc = 1.0 / std::max(ny, 1e-300);
    fe_sa::parallel_ranges(n, nt, [&](int64_t lo, int64_t hi, unsigned) {
      for (int64_t i = lo; i < hi; i++) x[i] = y[i] * sc;
    });
  }
  lam *= 1.1;
  if (!std::isfinite(lam) || lam <= 0.0) return fail(FE_ERR_ARG, "fe_sa_level_build: no spectral radius estimate");
  auto L = std::make_unique<fe_sa_level>();
  L->lam = lam;
  const double om = 4.0 / 3.0 / lam;
  // P = P0 - om D^-1 A P0
  fe_sa::build_rows(n, n_agg,
                    [&](int64_t i, fe_sa::Row &row) {
                      row.add(agg[i], 1.0);
                      const double s = -om / d[i];
                      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) row.add(agg[colidx[k]], s * vals[k]);
                    },
                    L->prp, L->pci, L->pv);
  // AP = A P
  std::vector<int32_t> aprp, apci;
  std::vector<double> apv;
  fe_sa::build_rows(n, n_agg,
                    [&](int64_t i, fe_sa::Row &row) {
                      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
                        const int32_t j = colidx[k];
                        const double a = vals[k];
                        for (int32_t q = L->prp[j]; q < L->prp[j + 1]; q++) row.add(L->pci[q], a * L->pv[q]);
                      }
                    },
                    aprp, apci, apv);
  // P^T: rows of P in ascending order within each column.  Each thread
  // counts its rows' entries per column, then writes them from its own
  // offset in each column (threads own ascending row ranges)
  std::vector<int32_t> trp((size_t)n_agg + 1, 0), tci(L->pci.size());
  std::vector<double> tv(L->pci.size());
  {
    std::vector<std::vector<int32_t>> pos(nt, std::vector<int32_t>((size_t)n_agg, 0));
    fe_sa::parallel_ranges(n, nt, [&](int64_t lo, int64_t hi, unsigned t) {
      std::vector<int32_t> &cnt = pos[t];
      for (int32_t q = L->prp[lo]; q < L->prp[hi]; q++) cnt[L->pci[q]]++;
    });
    for (int64_t c = 0; c < n_agg; c++) {
      int32_t at = trp[c];
      for (unsigned t = 0; t < nt; t++) {
        const int32_t k = pos[t][c];
        pos[t][c] = at;
        at += k;
      }
      trp[c + 1] = at;
    }
    fe_sa::parallel_ranges(n, nt, [&](int64_t lo, int64_t hi, unsigned t) {
      std::vector<int32_t> &at = pos[t];
      for (int64_t i = lo; i < hi; i++)
        for (int32_t q = L->prp[i]; q < L->prp[i + 1]; q++) {
          const int32_t w = at[L->pci[q]]++;
          tci[w] = (int32_t)i;
          tv[w] = L->pv[q];
        }
    });
  }
  // Ac = P^T (A P)
  fe_sa::build_rows(n_agg, n_agg,
                    [&](int64_t I, fe_sa::Row &row) {
                      for (int32_t q = trp[I]; q < trp[I + 1]; q++) {
                        const int32_t i = tci[q];
                        const double p = tv[q];
                        for (int32_t r = aprp[i]; r < aprp[i + 1]; r++) row.add(apci[r], p * apv[r]);
                      }
                    },
                    L->arp, L->aci, L->av);
  *out = L.release();
  return FE_OK;
}

int fe_sa_level_info(const fe_sa_level_t *L, int64_t *nnz_p, int64_t *nnz_ac, double *lam) {
  if (!L) return fail(FE_ERR_ARG, "fe_sa_level_info: null level");
  if (nnz_p) *nnz_p = (int64_t)L->pci.size();
  if (nnz_ac) *nnz_ac = (int64_t)L->aci.size();
  if (lam) *lam = L->lam;
  return FE_OK;
}

int fe_sa_level_copy(const fe_sa_level_t *L, int32_t *p_rowptr, int32_t *p_colidx, double *p_vals, int32_t *ac_rowptr,
                     int32_t *ac_colidx, double *ac_vals) {
  if (!L) return fail(FE_ERR_ARG, "fe_sa_level_copy: null level");
  if (p_rowptr) std::copy(L->prp.begin(), L->prp.end(), p_rowptr);
  if (p_colidx) std::copy(L->pci.begin(), L->pci.end(), p_colidx);
  if (p_vals) std::copy(L->pv.begin(), L->pv.end(), p_vals);
  if (ac_rowptr) std::copy(L->arp.begin(), L->arp.end(), ac_rowptr);
  if (ac_colidx) std::copy(L->aci.begin(), L->aci.end(), ac_colidx);
  if (ac_vals) std::copy(L->av.begin(), L->av.end(), ac_vals);
  return FE_OK;
}

void fe_sa_level_destroy(fe_sa_level_t *L) { delete L; }

int fe_csr_block(int64_t n, const int32_t *rowptr, const int32_t *colidx, const int8_t *label, int rl, int cl,
                 int64_t *nnz, int32_t *b_rowptr, int32_t *b_colidx, int64_t *b_slot) {
  if (n < 0 || !nnz || (n > 0 && (!rowptr || !colidx || !label)))
    return fail(FE_ERR_ARG, "fe_csr_block: null argument");
  // new numbers within each label, and the block's rows
  std::vector<int32_t> renum((size_t)std::max<int64_t>(n, 1));
  std::vector<int64_t> brows;
  int32_t c0 = 0, c1 = 0;
  for (int64_t i = 0; i < n; i++) {
    if (label[i] != 0 && label[i] != 1) return fail(FE_ERR_ARG, "fe_csr_block: labels must be 0 or 1");
    renum[i] = label[i] ? c1++ : c0++;
    if (label[i] == rl) brows.push_back(i);
  }
  const int64_t nb = (int64_t)brows.size();
  std::vector<int64_t> cnt((size_t)nb + 1, 0);
  const unsigned nt = fe_sa::threads_for(nb);
  fe_sa::parallel_ranges(nb, nt, [&](int64_t lo, int64_t hi, unsigned) {
    for (int64_t r = lo; r < hi; r++) {
      const int64_t i = brows[r];
      int64_t c = 0;
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++) c += label[colidx[k]] == cl;
      cnt[r + 1] = c;
    }
  });
  for (int64_t r = 0; r < nb; r++) cnt[r + 1] += cnt[r];
  *nnz = cnt[nb];
  if (!b_rowptr && !b_colidx && !b_slot) return FE_OK;
  if (!b_rowptr || !b_colidx || !b_slot) return fail(FE_ERR_ARG, "fe_csr_block: null output");
  if (cnt[nb] > 0x7fffffffLL) return fail(FE_ERR_ARG, "fe_csr_block: block exceeds int32 CSR");
  for (int64_t r = 0; r <= nb; r++) b_rowptr[r] = (int32_t)cnt[r];
  fe_sa::parallel_ranges(nb, nt, [&](int64_t lo, int64_t hi, unsigned) {
    std::vector<std::pair<int32_t, int64_t>> e;
    for (int64_t r = lo; r < hi; r++) {
      const int64_t i = brows[r];
      e.clear();
      for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++)
        if (label[colidx[k]] == cl) e.emplace_back(renum[colidx[k]], (int64_t)k);
      std::sort(e.begin(), e.end());
      int64_t at = cnt[r];
      for (const auto &x : e) {
        b_colidx[at] = x.first;
        b_slot[at++] = x.second;
      }
    }
  });
  return FE_OK;
}

} // extern "C"
