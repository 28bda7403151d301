// spread_layout_check.cu -- host-side check of the spread layout's index
// arithmetic (cmc_sweep.cuh / cmc_common.cuh), built and run by
// tests/test_spread_layout.py without a GPU.
//
// For random (nbeta, nseq, groups, R, N) within the host's launch
// constraints (groups of nseq/groups sequences or one more, N CTAs that hold
// the largest group at R replicas each and at most one per replica of the
// smallest), every group's layout over the N CTAs must
//   * hold every replica of the job exactly once over all groups,
//   * give each CTA 1..R replicas spanning at most two sequences of its group,
//   * give each sequence exactly one owner, whose own_r slot is the
//     sequence's ibeta = 0 replica, and
//   * count in own_ncta exactly the CTAs that hold replicas of the owned
//     sequence (the arrivals the owner waits for).
#include <algorithm>
#include <cstdio>
#include <vector>

#include "cmc_sweep.cuh"

using namespace cmc;

static unsigned long long g_x = 0x9E3779B97F4A7C15ull;
static int rnd(int lo, int hi)
{
  g_x ^= g_x << 13;
  g_x ^= g_x >> 7;
  g_x ^= g_x << 17;
  return lo + (int)(g_x % (unsigned long long)(hi - lo + 1));
}

#define CHECK(c)                                                                 \
  do {                                                                           \
    if (!(c)) {                                                                  \
      std::printf("FAIL %s: nbeta %d nseq %d groups %d R %d N %d group %d\n", #c, \
                  nbeta, nseq, ng, R, N, g);                                     \
      return 1;                                                                  \
    }                                                                            \
  } while (0)

int main()
{
  int cases = 0;
  for (int it = 0; it < 400000 && cases < 40000; ++it) {
    const int nbeta = rnd(1, 32), nseq = rnd(1, 80);
    const int ng = rnd(1, nseq), R = rnd(1, std::min(8, nbeta));
    const int rep_max = nbeta * ((nseq + ng - 1) / ng), rep_min = nbeta * (nseq / ng);
    const int Nlo = (rep_max + R - 1) / R;
    if (Nlo > rep_min) continue;
    const int N = rnd(Nlo, rep_min);
    std::vector<int> seen((size_t)nbeta * nseq, 0);
    int covered = 0, g = 0;
    for (g = 0; g < ng; ++g) {
      int seq0 = 0, n = 0;
      spread_group(nseq, ng, g, seq0, n);
      CHECK(seq0 == covered && n >= 1);
      covered += n;
      std::vector<int> holders(nseq, 0), owner(nseq, -1), ncta(nseq, 0);
      for (int b = 0; b < N; ++b) {
        const SpreadLayout L = make_spread_layout(nbeta, seq0, n, N, b, b * R);
        CHECK(L.cnt >= 1 && L.cnt <= R);
        CHECK(L.seq_lo >= seq0 && L.seq_hi < seq0 + n && L.seq_hi - L.seq_lo <= 1);
        CHECK(L.gstart >= seq0 * nbeta && L.gstart + L.cnt <= (seq0 + n) * nbeta);
        for (int f = L.gstart; f < L.gstart + L.cnt; ++f) {
          CHECK(f / nbeta >= L.seq_lo && f / nbeta <= L.seq_hi);
          ++seen[f];
        }
        for (int s = L.seq_lo; s <= L.seq_hi; ++s) ++holders[s];
        if (L.own >= 0) {
          CHECK(owner[L.own] < 0);
          owner[L.own] = b;
          ncta[L.own] = L.own_ncta;
          CHECK(L.own_r < L.cnt && L.gstart + L.own_r == L.own * nbeta);
        }
      }
      for (int s = seq0; s < seq0 + n; ++s) CHECK(owner[s] >= 0 && ncta[s] == holders[s]);
    }
    CHECK(covered == nseq);
    for (int f = 0; f < nbeta * nseq; ++f) CHECK(seen[f] == 1);
    ++cases;
  }
  std::printf("ok %d\n", cases);
  return cases > 0 ? 0 : 1;
}
