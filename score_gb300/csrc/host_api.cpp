// Host-only entry points of the C ABI: parameters (.uds), the host FP64 mobility
// weight.  Compiled into libscore_gb300.so and into the host-only libscore_host.so, which
// input preparation uses where the CUDA library must not be loaded (the CPU timing of
// the reference's algorithm); the synthetic-domain generator (host_generate.cpp) sits in
// both libraries the same way.
#include <cstdio>

#include "../../include/score_gb300.h"
#include "host_model.h"

extern "C" {

int score_params_default(score_params* out) {
    if (!out) return SCORE_ERR_ARG;
    score::params_default(out);
    return SCORE_OK;
}

int score_uds_read(const char* path, score_params* out) {
    if (!path || !out) return SCORE_ERR_ARG;
    char buf[512];
    const int s = score::uds_read(path, out, buf, sizeof buf);
    if (s != SCORE_OK) fprintf(stderr, "score_uds_read: %s\n", buf);
    return s;
}

int score_mobility_weight(const score_params* p, const double* rq, const double* dq, double* P) {
    if (!p || !rq || !dq || !P) return SCORE_ERR_ARG;
    *P = score::mobility_weight(*p, rq, dq);
    return SCORE_OK;
}

}  // extern "C"
