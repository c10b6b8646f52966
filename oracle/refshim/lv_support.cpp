// ORACLE (test infrastructure only): out-of-line helpers of the reference's utils module that its
// headers declare and the background subtraction path reaches (through lvAssert_/lvWarn and
// lv::Exception), written here instead of compiling modules/utils/src, which needs OpenCV.
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include <mutex>

#include "litiv/utils/cxx.hpp"

// printf-style formatting into a std::string
std::string lv::putf(const char* fmt, ...) {
    va_list a1, a2;
    va_start(a1, fmt);
    va_copy(a2, a1);
    const int n = std::vsnprintf(nullptr, 0, fmt, a1);
    va_end(a1);
    std::string s;
    if (n > 0) {
        std::vector<char> buf((size_t)n + 1);
        std::vsnprintf(buf.data(), buf.size(), fmt, a2);
        s.assign(buf.data(), (size_t)n);
    }
    va_end(a2);
    return s;
}

// the log mutex of the reference's thread-safe loggers
std::mutex& lv::getLogMutex() {
    static std::mutex m;
    return m;
}

// logging is silenced (the reference's default verbosity is 1): the bridge reports errors as status
// codes, and the tests run many instances
int lv::getVerbosity() { return -1; }
