// Host emulation of the line FFTs of cupss_gb300/csrc/fft.cuh: the M threads of one
// line run the device functions in turn, with a plain array as the transpose buffer,
// for every supported length, both directions and both forms (four-step, split).
// Checks against a direct DFT in double precision, and that every layout (step-1,
// step-2, transpose stores) is a permutation of the line's positions.  Built and run by tests/test_fft_layout.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "fft.cuh"

using namespace cupssgb;

static std::vector<float2> make_twiddles() {
  std::vector<float2> h(kTwLen);
  fill_twiddle_table(h.data());
  return h;
}

static bool is_perm(const std::vector<int>& seen) {
  for (int c : seen)
    if (c != 1) return false;
  return true;
}

template <int L, bool SP>
static int check(const float2* tw, unsigned seed) {
  using C = LineCfg<L, SP>;
  constexpr int M = C::M, R = C::R;
  static_assert(M * R == L, "threads x values = line length");
  int bad = 0;
  std::vector<float2> x(L), X(L), T(L), y(L);
  srand(seed);
  for (int n = 0; n < L; ++n)
    x[n] = make_float2((float)rand() / RAND_MAX - 0.5f, (float)rand() / RAND_MAX - 0.5f);
  // layouts are permutations
  std::vector<int> s1(L, 0), s2(L, 0), t1(L, 0), ti(L, 0);
  for (int m = 0; m < M; ++m)
    for (int i = 0; i < R; ++i) {
      s1[pos_step1<L, SP>(m, i)]++;
      s2[pos_step2<L, SP>(m, i)]++;
      t1[pos_t1<L, SP>(m, i)]++;
      if (pos_step2<L, SP>(m, i) != m + step2_off<L, SP>(i) || step2_off<L, SP>(i) % M != 0) bad++;
    }
  for (int m = 0; m < M; ++m) {
    float2 v[R] = {};
    inv_store_t<L, SP>(v, m, [&](int n, float2) { ti[n]++; });
  }
  if (!is_perm(s1) || !is_perm(s2) || !is_perm(t1) || !is_perm(ti)) {
    std::printf("L=%d: a layout is not a permutation\n", L);
    return 1;
  }
  // forward: step 1 of every thread, then step 2 of every thread
  for (int m = 0; m < M; ++m) {
    float2 v[R];
    for (int r = 0; r < R; ++r) v[r] = x[pos_step1<L, SP>(m, r)];
    fwd_step1<L, SP>(v, m, tw);
    for (int s = 0; s < R; ++s) T[pos_t1<L, SP>(m, s)] = v[s];
  }
  for (int m = 0; m < M; ++m) {
    float2 v[R];
    fwd_load_step2<L, SP>(v, m, tw, [&](int n) { return T[n]; });
    for (int i = 0; i < R; ++i) X[pos_step2<L, SP>(m, i)] = v[i];
  }
  double err = 0, ref = 0;
  for (int k = 0; k < L; ++k) {
    double re = 0, im = 0;
    for (int n = 0; n < L; ++n) {
      const double a = -2.0 * M_PI * (double)((long)n * k % L) / L;
      re += x[n].x * std::cos(a) - x[n].y * std::sin(a);
      im += x[n].x * std::sin(a) + x[n].y * std::cos(a);
    }
    err = std::fmax(err, std::hypot(X[k].x - re, X[k].y - im));
    ref = std::fmax(ref, std::hypot(re, im));
  }
  if (err > 1e-5 * std::fmax(ref, 1.0) * std::log2((double)L + 1)) {
    std::printf("L=%d forward: max error %.3e (max |X| %.3e)\n", L, err, ref);
    bad++;
  }
  // inverse of X: L * x
  for (int m = 0; m < M; ++m) {
    float2 v[R];
    for (int i = 0; i < R; ++i) v[i] = X[pos_step2<L, SP>(m, i)];
    inv_step2<L, SP>(v, m, tw);
    inv_store_t<L, SP>(v, m, [&](int n, float2 z) { T[n] = z; });
  }
  for (int m = 0; m < M; ++m) {
    float2 v[R];
    inv_load_step1<L, SP>(v, m, tw, [&](int n) { return T[n]; });
    for (int r = 0; r < R; ++r) y[pos_step1<L, SP>(m, r)] = v[r];
  }
  double ierr = 0;
  for (int n = 0; n < L; ++n)
    ierr = std::fmax(ierr, std::hypot(y[n].x / L - x[n].x, y[n].y / L - x[n].y));
  if (ierr > 1e-5 * std::log2((double)L + 1)) {
    std::printf("L=%d inverse: max error %.3e\n", L, ierr);
    bad++;
  }
  std::printf("L=%4d M=%3d R=%2d split=%d fwd %.2e inv %.2e\n", L, M, R, (int)C::kSplit, err / std::fmax(ref, 1.0),
              ierr);
  return bad;
}

int main() {
  const std::vector<float2> h = make_twiddles();
  const float2* tw = h.data();
  int bad = 0;
  bad += check<1, false>(tw, 1);
  bad += check<2, false>(tw, 2);
  bad += check<4, false>(tw, 3);
  bad += check<8, false>(tw, 4);
  bad += check<16, false>(tw, 5);
  bad += check<32, false>(tw, 6);
  bad += check<64, false>(tw, 7);
  bad += check<128, false>(tw, 8);
  bad += check<256, false>(tw, 9);
  bad += check<512, false>(tw, 10);
  bad += check<1024, false>(tw, 11);
  bad += check<256, true>(tw, 12);
  bad += check<512, true>(tw, 13);
  bad += check<1024, true>(tw, 14);
  // lengths 3 * 2^a: radix-3 butterflies in the register DFTs, J = R/M of 3 or 6
  bad += check<3, false>(tw, 15);
  bad += check<6, false>(tw, 16);
  bad += check<12, false>(tw, 17);
  bad += check<24, false>(tw, 18);
  bad += check<48, false>(tw, 19);
  bad += check<96, false>(tw, 20);
  bad += check<192, false>(tw, 21);
  bad += check<384, false>(tw, 22);
  for (int L = 1; L <= 1024; L *= 2)
    if (line_m_of(L, false) <= 0 || line_m_of(L, true) <= 0) bad++;
  if (line_m_of(96, false) != LineCfg<96>::M || line_m_of(192, true) != LineCfg<192, true>::M ||
      line_m_of(384, false) != LineCfg<384>::M || line_m_of(3, false) != LineCfg<3>::M)
    bad++;
  if (line_m_of(512, true) != LineCfg<512, true>::M || line_m_of(1024, true) != LineCfg<1024, true>::M ||
      line_m_of(1024, false) != LineCfg<1024>::M || line_m_of(64, true) != LineCfg<64>::M)
    bad++;
  std::printf(bad ? "FAILED\n" : "OK\n");
  return bad ? 1 : 0;
}
