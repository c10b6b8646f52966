/* ORACLE (test infrastructure only): routes the reference's rand() calls to the counter-based
 * generator that the GPU path and the C restatement use. Force-included (g++ -include) before
 * every reference source compiled into oracle/_ref/libref.so.
 *
 * Every rand() of the reference becomes draw k of pixel p in frame t:
 *     block = philox4x32-10(ctr = {k>>2, p, t, 0}, key = {seed_lo, seed_hi})
 *     draw  = block[k & 3] & 0x7fffffff     (31 bits, like glibc's RAND_MAX)
 * The pixel comes from the name `nPxIter`: inside the reference's pixel loops a local
 * `const size_t nPxIter` holds the raster index of the pixel being processed and shadows the
 * namespace-scope sentinel below, so `rand()` there is attributed to that pixel; a draw outside any
 * pixel loop (the refresh start position, BackgroundSubtractorSuBSENSE.cpp:86) sees the sentinel
 * and is a frame-level draw (p = 0xffffffff). The frame t is the instance's m_nFrameIdx (read through
 * a pointer at each draw) and the per-pixel counters restart at 0 when the bridge starts a frame
 * (initialize() and every apply()). The generator state is per host thread (one instance runs on
 * one thread at a time).
 */
#ifndef LV_ORACLE_SHIM_RAND_H
#define LV_ORACLE_SHIM_RAND_H

/* every standard header that might name rand() is parsed before the macro exists */
#include <stdlib.h>
#include <cstdlib>
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <climits>
#include <cfloat>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <deque>
#include <exception>
#include <fstream>
#include <functional>
#include <future>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <queue>
#include <random>
#include <ratio>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>
#include <cinttypes>

/* draw attributed to raster pixel `px` (SIZE_MAX: a frame-level draw) */
int lvshim_rand(size_t px);

/* the frame-level sentinel, shadowed by the reference's per-pixel `nPxIter` locals */
static const size_t nPxIter = SIZE_MAX;

#define rand() lvshim_rand(nPxIter)

#endif
