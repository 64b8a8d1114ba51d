// Test harness for pfdd::ConvergeTracker (the host-side convergence test of the
// whole-step contexts and the server), built by tests/test_converge_cpu.py with
// the host compiler.  Input on stdin: gamma_prev, then the number of steps,
// then one gamma per step (any strtod form; the test writes C99 hex floats so
// that every double arrives exactly).  Output: one line per step,
// "<min_steps before the step> <1 if the tracker stops after it, else 0>".
// The tracker is not reset at a stop: the lines after one show how it goes on.
#include <cstdio>
#include <cstdlib>

#include "pfdd_converge.h"

static bool read_double(double *v) {
  char buf[128];
  if (std::scanf("%127s", buf) != 1) return false;
  char *end = nullptr;
  *v = std::strtod(buf, &end);
  return end != buf && *end == '\0';
}

int main() {
  double prev = 0.0, g = 0.0;
  long long n = 0;
  if (!read_double(&prev) || std::scanf("%lld", &n) != 1 || n < 0) return 2;
  pfdd::ConvergeTracker t;
  t.reset(prev);
  for (long long i = 0; i < n; ++i) {
    if (!read_double(&g)) return 3;
    const int k = t.min_steps();
    const bool stop = t.update(g);
    std::printf("%d %d\n", k, stop ? 1 : 0);
  }
  return 0;
}
