/* Test infrastructure only. The reference seeds every random stream with time(NULL)
 * (src/simulation/cells_population.cu:34, src/simulation/proliferation.cu:242). Preloaded
 * into the reference binary, this returns PROCELL_REF_TIME instead, so that each run of a
 * distribution check gets its own, recorded seed without sleeping between runs. */
#include <stdlib.h>
#include <time.h>

time_t time(time_t* t) {
  const char* s = getenv("PROCELL_REF_TIME");
  time_t v = s ? (time_t)strtoll(s, NULL, 10) : (time_t)0;
  if (t) *t = v;
  return v;
}
