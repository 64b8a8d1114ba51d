// pfdd_converge.h -- the inner loop's convergence test (plasticconverge,
// PFDD_Final_GPU.c:3732-3785, applied by the do-while of F:4574-4691) as a
// host-side tracker: the whole-step contexts (pfdd_step_converge*) keep one a
// replica, the server one a solve.
#pragma once
#include <cstdint>
#include <vector>

namespace pfdd {

// The state of one inner loop's test: which of its steps passed, the count of
// passing steps with a full window behind, the loop's step count and the
// previous gamma.
struct ConvergeTracker {
  std::vector<uint8_t> test;
  int count = 0, it = 0;
  double last = 0.0;

  // starts a loop (F:4567-4572); gamma_prev is the gamma its first step is
  // compared with (the last gamma of the previous loop, 0.0 before the first)
  void reset(double gamma_prev) {
    test.clear();
    count = 0;
    it = 0;
    last = gamma_prev;
  }

  // The gamma of one more step: the step passes when gamma changed by less
  // than 1e-8 relative (1e-15 absolute when gamma is 0) or |gamma| < 1e-12
  // (1e-14); a passing step whose last 30 steps all passed adds one to the
  // count, one whose window is not full resets it (a failing step leaves it);
  // the loop stops when the count reaches 5.  True: the loop stops after
  // this step.
  bool update(double g) {
    bool passed;
    if (g != 0) {
      const double r = (g - last) / g;
      passed = (r < 0 ? -r : r) < 1E-8 || (g > 0 ? g : -g) < 1E-12;
    } else {
      const double d = g - last;
      passed = (d < 0 ? -d : d) < 1E-15 || (g > 0 ? g : -g) < 1E-14;
    }
    if ((int)test.size() <= it) test.resize((size_t)it + 1, 0);
    if (passed) {
      test[it] = 1;
      if (it >= 29) {
        int t = 0;
        for (int i = 0; i < 30; ++i) t += test[it - i];
        if (t == 30) count++;
        else if (count != 0) count = 0;
      }
    }
    bool stop = false;
    if (count == 5) {
      count++;
      stop = true;
    }
    last = g;
    it++;
    return stop;
  }

  // The fewest further steps after which the loop can stop: with a run of r
  // passing steps behind and the count at k, every step passing from here on,
  // 5 - k steps when the window is already full (r >= 29, k < 5), else 29 - r
  // steps to fill it and 5 to count (a count past 5, after a stop, must first
  // be reset: a failing step and 34 more).  Chunks of steps no longer than
  // this end at a stop at the earliest, never run past one.
  int min_steps() const {
    int r = 0;
    while (r < 29 && r < it && test[it - 1 - r]) ++r;
    if (r >= 29) return count < 5 ? 5 - count : 35;
    return 34 - r;
  }
};

}  // namespace pfdd
