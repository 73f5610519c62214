// Host-side construction of the bitmask transformation cost matrix,
// restating Cost_matrix.Two_D (cost_matrix.ml) for the combinations case
// (DNA: A, C, G, T and gap as five bits, 31 non-empty sets).
#include <cstring>
#include <algorithm>
#include "poyd_internal.h"

namespace {

constexpr int kMaxInt = 1073741823;  // cost_matrix.ml:39 (Int32.max_int lsr 1)

inline int idx(int a, int b) { return (a << 5) + b; }
inline bool single(int x) { return x && !(x & (x - 1)); }

template <class F>
void for_bits(int set, F f) {
  for (int bit = 1; bit <= 16; bit <<= 1)
    if (set & bit) f(bit);
}

// fill_best_cost_and_median_for_all_combinations (cost_matrix.ml:323-354)
void fill_via_intermediate(poyd_cm &m) {
  for (int i = 1; i < 32; ++i)
    for (int j = 1; j < 32; ++j) {
      int best = 0, c = kMaxInt, w = 0;
      for_bits(i, [&](int a) {
        for_bits(j, [&](int b) {
          for (int k = 0; k < 5; ++k) {
            const int v = 1 << k;
            const int goa = (m.cost_model == 1 && v == m.gap && (a & m.gap) && (b & m.gap))
                                ? m.gap_open : 0;
            const int tc = m.cost[idx(a, v)] + m.cost[idx(v, b)] + goa;
            if (tc < c) { c = tc; best = v; }
            else if (tc == c) best |= v;
          }
          w = std::max(w, m.cost[idx(a, b)]);
        });
      });
      if (single(i) && single(j)) {
        m.median[idx(i, j)] = uint8_t(i | j);
      } else {
        m.cost[idx(i, j)] = c;
        // cleanup (cost_matrix.ml:246-255): identity unless already affine
        if (m.cost_model == 1 && best != m.gap && (best & m.gap)) best = m.gap;
        m.median[idx(i, j)] = uint8_t(best);
      }
      m.worst[idx(i, j)] = w;
    }
}

// fill_best_cost_and_median_for_all_combinations_bitwise (cost_matrix.ml:270-321)
void fill_bitwise(poyd_cm &m) {
  for (int i = 1; i < 32; ++i)
    for (int j = 1; j < 32; ++j) {
      if (single(i) && single(j)) {
        m.median[idx(i, j)] = uint8_t(i | j);
        m.worst[idx(i, j)] = m.cost[idx(i, j)];
        continue;
      }
      int best = kMaxInt, med = 0, worst = 0;
      auto scan = [&](int x, int y) {
        for_bits(x, [&](int a) {
          for_bits(y, [&](int b) {
            const int c = m.cost[idx(a, b)];
            if (c < best) { best = c; med = a | b; }
            else if (c == best) med |= a | b;
            worst = std::max(worst, c);
          });
        });
      };
      scan(j, i);
      scan(i, j);
      if (i & j) {
        m.median[idx(i, j)] = uint8_t(i & j);
        m.cost[idx(i, j)] = 0;
      } else {
        m.median[idx(i, j)] = uint8_t(med);
        m.cost[idx(i, j)] = best;
      }
      m.worst[idx(i, j)] = worst;
    }
}

// fill_default_prepend_tail (cost_matrix.ml:397-403)
void fill_prepend_tail(poyd_cm &m) {
  m.tail[0] = m.prepend[0] = 0;
  for (int i = 1; i < 32; ++i) {
    m.tail[i] = m.cost[idx(i, m.gap)];
    m.prepend[i] = m.cost[idx(m.gap, i)];
  }
}

// input_is_metric (cost_matrix.ml:512-517)
bool metric5(const int32_t *l) {
  for (int i = 0; i < 25; ++i) if (l[i] < 0) return false;
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      if (l[i * 5 + j] != l[j * 5 + i]) return false;
      for (int k = 0; k < 5; ++k)
        if (l[i * 5 + j] > l[i * 5 + k] + l[k * 5 + j]) return false;
    }
  for (int i = 0; i < 5; ++i) if (l[i * 5 + i] != 0) return false;
  return true;
}

}  // namespace

extern "C" int poyd_cm_of_matrix5(poyd_cm *m, const int32_t *mat25, int32_t gap_open) {
  if (!m || !mat25) return poyd::fail(POYD_EINVAL, "poyd_cm_of_matrix5: null argument");
  std::memset(m, 0, sizeof(*m));
  m->gap = 16; m->a_sz = 31; m->lcm = 5; m->combinations = 1; m->all_elements = 31;
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) m->cost[idx(1 << i, 1 << j)] = mat25[i * 5 + j];
  if (metric5(mat25)) { m->is_metric = 1; fill_via_intermediate(*m); }
  else fill_bitwise(*m);
  fill_prepend_tail(*m);
  if (gap_open >= 0) {
    m->cost_model = 1;
    m->gap_open = gap_open;
    fill_bitwise(*m);
    fill_prepend_tail(*m);
  }
  return POYD_OK;
}

extern "C" int poyd_cm_dna(poyd_cm *m, int32_t sub, int32_t indel, int32_t gap_open) {
  int32_t l[25];
  for (int x = 0; x < 5; ++x)
    for (int y = 0; y < 5; ++y)
      l[x * 5 + y] = (x == y) ? 0 : ((x == 4 || y == 4) ? indel : sub);
  return poyd_cm_of_matrix5(m, l, gap_open);
}
