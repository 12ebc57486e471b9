// Host side of the FFT plans and the library-wide error string.
#include <cmath>
#include <cstdarg>
#include <vector>

#include "fft.cuh"

namespace mrsr {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}
const char* get_error() { return g_last_error.c_str(); }

bool build_radices(int L, int* radix, int* nstages) {
  if (L < 1) return false;
  int a = 0, b = 0, c = 0, r = L;
  while (r % 2 == 0) { r /= 2; ++a; }
  while (r % 3 == 0) { r /= 3; ++b; }
  while (r % 5 == 0) { r /= 5; ++c; }
  if (r != 1) return false;
  std::vector<int> p2;
  while (a >= 3) { p2.push_back(8); a -= 3; }
  if (a == 2) p2.push_back(4);
  if (a == 1) p2.push_back(2);
  std::vector<int> odd;
  for (int i = 0; i < b; ++i) odd.push_back(3);
  for (int i = 0; i < c; ++i) odd.push_back(5);
  std::vector<int> out;
  if (p2.size() >= 2) {
    out.push_back(p2.front());
    for (size_t i = 1; i + 1 < p2.size(); ++i) out.push_back(p2[i]);
    for (int o : odd) out.push_back(o);
    out.push_back(p2.back());
  } else {
    for (int x : p2) out.push_back(x);
    for (int o : odd) out.push_back(o);
  }
  if (L == 1) out.clear();
  if ((int)out.size() > kMaxStages) return false;
  *nstages = (int)out.size();
  for (size_t i = 0; i < out.size(); ++i) radix[i] = out[i];
  return true;
}

int FftPlanHost::init(int L) {
  plan = FftPlan();
  plan.L = L;
  MRSR_REQUIRE(build_radices(L, plan.radix, &plan.nstages), MRSR_ERR_ARG,
               "FFT length %d is not composed of the prime factors 2, 3 and 5", L);
  std::vector<float2> h(L);
  for (int p = 0; p < L; ++p) {
    // exp(-2 pi i p / L) evaluated in double precision
    double ang = -2.0 * M_PI * (double)p / (double)L;
    h[p] = make_float2((float)std::cos(ang), (float)std::sin(ang));
  }
  MRSR_TRY(tw.alloc(sizeof(float2) * L));
  MRSR_TRY(copy_h2d(tw.p, h.data(), sizeof(float2) * L));
  plan.tw = tw.as<float2>();
  return MRSR_OK;
}

}  // namespace mrsr

extern "C" const char* mrsr_last_error(void) { return mrsr::get_error(); }
extern "C" int mrsr_version(void) { return 100; }
