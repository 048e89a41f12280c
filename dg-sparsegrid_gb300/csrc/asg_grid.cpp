// Sparse-grid element tables, 1-D index maps and element-pair connectivity.
//
// Host C++ restatement of the reference's setup-time index structures; the results are
// bit-identical to hash_table_sparse_nD.m / hash_table_nD.m / connect_nD.m (tested against
// the reference's gold files).  They feed the plan's idx1d and pair lists.
#include <algorithm>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "asg_internal.h"

namespace {

using Tuple = std::vector<int>;

// Level tuples with sum == s, t[k] <= levmax[k], enumerated with the last dimension
// slowest and ascending (perm_eq_d.m:45-80 with last_index_decreasing = 0).
void perm_eq_d(int idim, const int* levmax, int s, std::vector<Tuple>& out, Tuple& cur) {
  if (idim == 1) {
    if (levmax[0] >= s) {
      cur[0] = s;
      out.push_back(cur);
    }
    return;
  }
  const int hi = std::min(levmax[idim - 1], s);
  for (int il = 0; il <= hi; ++il) {
    cur[idim - 1] = il;
    perm_eq_d(idim - 1, levmax, s - il, out, cur);
  }
}

// Full-grid tuples t[k] <= levmax[k], last dimension slowest (perm_max.m).
void perm_max(int idim, const int* levmax, std::vector<Tuple>& out, Tuple& cur) {
  if (idim == 0) {
    out.push_back(cur);
    return;
  }
  for (int i = 0; i <= levmax[idim - 1]; ++i) {
    cur[idim - 1] = i;
    perm_max(idim - 1, levmax, out, cur);
  }
}

// Tuples with sum <= n, last dimension slowest (perm_leq.m, order_by_n = 0).
void perm_leq(int idim, int n, std::vector<Tuple>& out, Tuple& cur) {
  if (idim == 1) {
    for (int v = 0; v <= n; ++v) {
      cur[0] = v;
      out.push_back(cur);
    }
    return;
  }
  for (int i = 0; i <= n; ++i) {
    cur[idim - 1] = i;
    perm_leq(idim - 1, n - i, out, cur);
  }
}

inline long long idx1d_of(int lev, int cell) { return lev == 0 ? 1 : (1LL << (lev - 1)) + cell + 1; }

// Append the cells of one level tuple, dimension 1 fastest (lev_cell_to_1D_index_set.m).
void append_cells(const Tuple& lev, std::vector<int>& levels, std::vector<int>& cells) {
  const int d = static_cast<int>(lev.size());
  std::vector<int> size(d), c(d, 0);
  long long total = 1;
  for (int k = 0; k < d; ++k) {
    size[k] = 1 << std::max(0, lev[k] - 1);
    total *= size[k];
  }
  for (long long n = 0; n < total; ++n) {
    for (int k = 0; k < d; ++k) {
      levels.push_back(lev[k]);
      cells.push_back(c[k]);
    }
    for (int k = 0; k < d; ++k) {
      if (++c[k] < size[k]) break;
      c[k] = 0;
    }
  }
}

asg_status emit_table(int d, const std::vector<Tuple>& ptable, int max_lev, int* levels, int* cells,
                      unsigned long long* keys, long long capacity, long long* count) {
  std::vector<int> lv, cl;
  for (const auto& t : ptable) append_cells(t, lv, cl);
  const long long n = static_cast<long long>(lv.size()) / d;
  if (count) *count = n;
  if (capacity == 0) return ASG_OK;
  if (capacity < n) return asg::fail(ASG_ERR_CAPACITY, "element table needs %lld entries, capacity %lld", n, capacity);
  for (long long e = 0; e < n; ++e) {
    unsigned long long key = 0, stride = 1;
    for (int k = 0; k < d; ++k) {
      if (levels) levels[e * d + k] = lv[e * d + k];
      if (cells) cells[e * d + k] = cl[e * d + k];
      if (max_lev >= 0) {
        key += static_cast<unsigned long long>(idx1d_of(lv[e * d + k], cl[e * d + k]) - 1) * stride;
        stride <<= max_lev;
      }
    }
    if (keys) keys[e] = key;
  }
  return ASG_OK;
}

// connect_1D.m: 2^Lev x 2^Lev 0/1 matrix of 0-based 1-D indices.
std::vector<uint8_t> connect_1d(int Lev) {
  const int n = 1 << Lev;
  std::vector<uint8_t> C(static_cast<size_t>(n) * n, 0);
  auto id = [](int l, int c) { return static_cast<int>(idx1d_of(l, c) - 1); };
  auto set = [&](int i, int j) {
    C[static_cast<size_t>(i) * n + j] = 1;
    C[static_cast<size_t>(j) * n + i] = 1;
  };
  for (int Lx = 0; Lx <= Lev; ++Lx) {
    const int ncx = 1 << std::max(0, Lx - 1);
    for (int Px = 0; Px < ncx; ++Px) {
      const int I = id(Lx, Px);
      for (int q = std::max(Px - 1, 0); q <= std::min(Px + 1, ncx - 1); ++q) set(I, id(Lx, q));
      if (Px == 0)
        set(I, id(Lx, ncx - 1));
      else if (Px == ncx - 1)
        set(I, id(Lx, 0));
      for (int Ly = Lx + 1; Ly <= Lev; ++Ly) {
        const int nL = Ly - Lx;
        const int ncy = 1 << (Ly - 1);
        int lo, hi;
        if (Lx > 0) {
          lo = std::max((1 << nL) * Px - 1, 0);
          hi = std::min((1 << nL) * Px + (1 << nL), ncy - 1);
        } else {
          lo = std::max((1 << (nL - 1)) * Px - 1, 0);
          hi = std::min((1 << (nL - 1)) * Px + (1 << (nL - 1)), ncy - 1);
        }
        set(I, id(Ly, 0));
        for (int q = lo; q <= hi; ++q) set(I, id(Ly, q));
        set(I, id(Ly, (1 << std::max(0, Ly - 1)) - 1));
      }
    }
  }
  return C;
}

}  // namespace

extern "C" {

asg_status asg_hash_table_sparse_nd(int num_dims, const int* lev_vec, int max_lev, int grid, int* levels, int* cells,
                                    unsigned long long* keys, long long capacity, long long* count) {
  if (num_dims < 1 || num_dims > asg::kMaxDims || !lev_vec)
    return asg::fail(ASG_ERR_INVALID, "hash_table_sparse_nD: num_dims=%d out of range", num_dims);
  int lmax = 0;
  for (int k = 0; k < num_dims; ++k) {
    if (lev_vec[k] < 0 || lev_vec[k] > 30) return asg::fail(ASG_ERR_INVALID, "hash_table_sparse_nD: bad level");
    if (lev_vec[k] > max_lev) return asg::fail(ASG_ERR_INVALID, "hash_table_sparse_nD: lev %d > max_lev %d", lev_vec[k], max_lev);
    lmax = std::max(lmax, lev_vec[k]);
  }
  if (static_cast<long long>(max_lev) * num_dims > 64)
    return asg::fail(ASG_ERR_UNSUPPORTED, "hash_table_sparse_nD: keys overflow 64 bits (max_lev*d=%d)", max_lev * num_dims);
  std::vector<Tuple> ptable;
  Tuple cur(num_dims, 0);
  if (grid == ASG_GRID_SG) {
    for (int s = lmax; s >= 0; --s) perm_eq_d(num_dims, lev_vec, s, ptable, cur);
  } else if (grid == ASG_GRID_FG) {
    perm_max(num_dims, lev_vec, ptable, cur);
  } else {
    return asg::fail(ASG_ERR_INVALID, "hash_table_sparse_nD: unknown grid type %d", grid);
  }
  return emit_table(num_dims, ptable, max_lev, levels, cells, keys, capacity, count);
}

asg_status asg_hash_table_nd(int num_dims, int lev, int grid, int* levels, int* cells, long long capacity,
                             long long* count) {
  if (num_dims < 1 || num_dims > asg::kMaxDims || lev < 0 || lev > 30)
    return asg::fail(ASG_ERR_INVALID, "hash_table_nD: bad num_dims=%d / lev=%d", num_dims, lev);
  std::vector<Tuple> ptable;
  Tuple cur(num_dims, 0);
  if (grid == ASG_GRID_SG) {
    perm_leq(num_dims, lev, ptable, cur);
  } else if (grid == ASG_GRID_FG) {
    std::vector<int> lm(num_dims, lev);
    perm_max(num_dims, lm.data(), ptable, cur);
  } else {
    return asg::fail(ASG_ERR_INVALID, "hash_table_nD: unknown grid type %d", grid);
  }
  return emit_table(num_dims, ptable, -1, levels, cells, nullptr, capacity, count);
}

asg_status asg_element_idx1d(int num_dims, long long num_elems, const int* levels, const int* cells, int* idx1d) {
  if (num_dims < 1 || num_elems < 0 || (num_elems > 0 && (!levels || !cells || !idx1d)))
    return asg::fail(ASG_ERR_INVALID, "element_idx1d: bad arguments");
  for (long long i = 0; i < num_elems * num_dims; ++i) {
    if (levels[i] < 0 || levels[i] > 30 || cells[i] < 0 || cells[i] >= (1 << std::max(0, levels[i] - 1)))
      return asg::fail(ASG_ERR_INVALID, "element_idx1d: (lev=%d, cell=%d) invalid at %lld", levels[i], cells[i], i);
    idx1d[i] = static_cast<int>(idx1d_of(levels[i], cells[i]));
  }
  return ASG_OK;
}

asg_status asg_connect_nd(int num_dims, long long num_elems, const int* levels, const int* cells, int levsum,
                          int levmax, int grid, long long* row_ptr, int* cols, long long capacity,
                          long long* num_pairs) {
  if (num_dims < 1 || num_dims > asg::kMaxDims || num_elems < 0 || levsum < 0 || levmax < 0 || levmax > 20 ||
      (num_elems > 0 && (!levels || !cells)))
    return asg::fail(ASG_ERR_INVALID, "connect_nD: bad arguments");
  const int Lev = std::max(levsum, levmax);
  if (Lev > 14) return asg::fail(ASG_ERR_UNSUPPORTED, "connect_nD: level %d too large for the dense 1-D table", Lev);
  const int n1 = 1 << Lev;
  const std::vector<uint8_t> C = connect_1d(Lev);
  std::vector<int> lev1(n1), cell1(n1);
  for (int Lx = 0, k = 0; Lx <= Lev; ++Lx)
    for (int Px = 0; Px < (1 << std::max(0, Lx - 1)); ++Px, ++k) {
      lev1[k] = Lx;
      cell1[k] = Px;
    }
  // element lookup keyed by the 1-D index tuple
  std::unordered_map<unsigned long long, int> lookup;
  lookup.reserve(static_cast<size_t>(num_elems) * 2);
  std::vector<int> idx(static_cast<size_t>(num_elems) * num_dims);
  for (long long e = 0; e < num_elems; ++e) {
    unsigned long long key = 0;
    for (int k = 0; k < num_dims; ++k) {
      const int l = levels[e * num_dims + k], c = cells[e * num_dims + k];
      if (l < 0 || l > Lev || c < 0 || c >= (1 << std::max(0, l - 1)))
        return asg::fail(ASG_ERR_INVALID, "connect_nD: element %lld has (lev=%d, cell=%d) outside level %d", e, l, c, Lev);
      idx[e * num_dims + k] = static_cast<int>(idx1d_of(l, c) - 1);
      key = key * static_cast<unsigned long long>(n1) + static_cast<unsigned long long>(idx[e * num_dims + k]);
    }
    lookup.emplace(key, static_cast<int>(e));
  }
  std::vector<long long> rp(num_elems + 1, 0);
  std::vector<int> out;
  std::vector<std::vector<int>> lists(num_dims);
  std::vector<int> row;
  for (long long e = 0; e < num_elems; ++e) {
    for (int k = 0; k < num_dims; ++k) {
      lists[k].clear();
      const uint8_t* crow = &C[static_cast<size_t>(idx[e * num_dims + k]) * n1];
      for (int j = 0; j < n1; ++j)
        if (crow[j] && lev1[j] <= levmax) lists[k].push_back(j);
    }
    // enumerate the tuple product under the level-sum (SG) rule (index_leq_max.m / index_max.m)
    row.clear();
    std::vector<int> pos(num_dims, 0);
    bool done = false;
    for (int k = 0; k < num_dims; ++k)
      if (lists[k].empty()) done = true;
    while (!done) {
      int lsum = 0;
      unsigned long long key = 0;
      for (int k = 0; k < num_dims; ++k) {
        const int j = lists[k][pos[k]];
        lsum += lev1[j];
        key = key * static_cast<unsigned long long>(n1) + static_cast<unsigned long long>(j);
      }
      if (grid == ASG_GRID_FG || lsum <= levsum) {
        auto it = lookup.find(key);
        if (it == lookup.end())
          return asg::fail(ASG_ERR_INVALID, "connect_nD: connected element of %lld missing from the table", e);
        row.push_back(it->second);
      }
      int k = 0;
      while (k < num_dims && ++pos[k] == static_cast<int>(lists[k].size())) pos[k++] = 0;
      if (k == num_dims) done = true;
    }
    std::sort(row.begin(), row.end());
    rp[e + 1] = rp[e] + static_cast<long long>(row.size());
    out.insert(out.end(), row.begin(), row.end());
  }
  if (num_pairs) *num_pairs = rp[num_elems];
  if (capacity == 0) return ASG_OK;
  if (capacity < rp[num_elems])
    return asg::fail(ASG_ERR_CAPACITY, "connect_nD needs %lld pairs, capacity %lld", rp[num_elems], capacity);
  if (!row_ptr || !cols) return asg::fail(ASG_ERR_INVALID, "connect_nD: null output");
  std::copy(rp.begin(), rp.end(), row_ptr);
  std::copy(out.begin(), out.end(), cols);
  return ASG_OK;
}

}  // extern "C"
