// Wall-clock timer with the reference's interface (lib/timer.h).
#ifndef DS_GB300_CXX_TIMER_H
#define DS_GB300_CXX_TIMER_H

#include <cstddef>
#include <sys/time.h>

typedef struct timeval tv;

class Timer {
 public:
  Timer();
  static tv get_time();
  static double interval(const tv t0, const tv t1);
  void reset();
  double elapsed() const;

 private:
  tv t0;
};

extern Timer total_timer;

#endif
