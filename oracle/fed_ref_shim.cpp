// C entry point over the reference's own src/lib/fed.cpp (compiled in place
// from the reference tree by oracle/Makefile, target "ref"), used only to pin
// the oracle's FED schedule.  Test infrastructure.
#include <vector>
#include "fed.h"

extern "C" int fedref_tau_by_process_time(float T, int M, float tau_max, int reordering, float *tau, int cap)
{
  std::vector<float> v;
  const int n = fed_tau_by_process_time(T, M, tau_max, reordering != 0, v);
  for (int i = 0; i < n && i < cap; i++) tau[i] = v[i];
  return n;
}

extern "C" int fedref_is_prime(int number) { return fed_is_prime_internal(number) ? 1 : 0; }
