// Host-side parallel loops (OpenMP) of the build: prefix sums and stable
// partitions over the millions of far blocks of an operator or a batch.
#pragma once

#include <omp.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

namespace hodlr {

// Threads for a pass over n items: one below 2^16 items, else up to the
// OpenMP pool.
inline int par_threads(int64_t n) {
  if (n < (int64_t(1) << 16)) return 1;
  return std::max(1, std::min<int>(omp_get_max_threads(), int(n >> 14)));
}

// The contiguous share [b, e) of thread t of T over n items.
inline void par_share(int64_t n, int t, int T, int64_t& b, int64_t& e) {
  b = n * t / T;
  e = n * (t + 1) / T;
}

// out[0] = 0, out[i + 1] = out[i] + f(i) for i < n (out has n + 1 entries).
template <class F>
void par_exclusive_scan(int64_t n, uint64_t* out, F f) {
  const int T = par_threads(n);
  std::vector<uint64_t> part(size_t(T) + 1, 0);
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num();
    int64_t b, e;
    par_share(n, t, T, b, e);
    uint64_t s = 0;
    for (int64_t i = b; i < e; i++) {
      out[i + 1] = s;  // local prefix, made global below
      s += f(i);
    }
    part[size_t(t) + 1] = s;
#pragma omp barrier
#pragma omp single
    for (int k = 0; k < T; k++) part[size_t(k) + 1] += part[size_t(k)];
    const uint64_t base = part[size_t(t)];
    for (int64_t i = b; i < e; i++) out[i + 1] = base + out[i + 1] + f(i);
  }
  out[0] = 0;
}

// Running offsets within groups: for i < n in order, off[i] = the sum of
// size(k) over earlier k with group(k) == group(i); total[g] = the sum over
// group g (groups 0 .. ngroups - 1).
template <class G, class S>
void par_group_offsets(int64_t n, int ngroups, uint64_t* off, std::vector<uint64_t>& total, G group, S size) {
  const int T = par_threads(n);
  std::vector<uint64_t> acc(size_t(T) * size_t(ngroups), 0);
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num();
    int64_t b, e;
    par_share(n, t, T, b, e);
    uint64_t* a = acc.data() + size_t(t) * size_t(ngroups);
    for (int64_t i = b; i < e; i++) a[group(i)] += size(i);
#pragma omp barrier
#pragma omp single
    {
      total.assign(size_t(ngroups), 0);
      for (int g = 0; g < ngroups; g++)
        for (int k = 0; k < T; k++) {
          const uint64_t v = acc[size_t(k) * size_t(ngroups) + size_t(g)];
          acc[size_t(k) * size_t(ngroups) + size_t(g)] = total[size_t(g)];
          total[size_t(g)] += v;
        }
    }
    for (int64_t i = b; i < e; i++) {
      const int g = group(i);
      off[i] = a[g];
      a[g] += size(i);
    }
  }
}

}  // namespace hodlr
