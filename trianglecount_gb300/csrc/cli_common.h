// cli_common.h -- helpers shared by libtc's command-line tools (C ABI only).
#pragma once

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "tc.h"

namespace cli {

inline double now_s() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

// Prints the library's last error and exits with status 1.
[[noreturn]] inline void die(const char *what, int st) {
    fprintf(stderr, "%s: %s: %s\n", what, tc_status_string(st), tc_last_error());
    exit(1);
}

#define CLI_CHECK(call)                          \
    do {                                         \
        int cli_st_ = (call);                    \
        if (cli_st_ != TC_OK) cli::die(#call, cli_st_); \
    } while (0)

// A file's integers in reading order, with a cursor.
struct Ints {
    uint64_t *v = nullptr;
    int64_t n = 0, pos = 0;
    ~Ints() { tc_host_free(v); }
    bool take(int64_t k, const uint64_t **out) {
        if (k < 0 || pos + k > n) return false;
        *out = v + pos;
        pos += k;
        return true;
    }
    bool next(uint64_t *x) {
        const uint64_t *p;
        if (!take(1, &p)) return false;
        *x = *p;
        return true;
    }
};

inline bool file_exists(const char *path) {
    FILE *f = fopen(path, "r");
    if (!f) return false;
    fclose(f);
    return true;
}

}  // namespace cli
