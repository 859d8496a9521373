/* Hooks linked into the staged reference build (oracle/_ref/rad_ref*).
 * ORACLE / TEST INFRASTRUCTURE ONLY: the product never links this.
 *
 * Environment (all optional):
 *   RAD_DUMP=path       at exit, write every slot of TriStore[0..trinum) in the
 *                       RADDUMP1 binary format read by oracle/raddump.py
 *   RAD_TRACE=path      one line per shooter step: "<n> <idx...>" (the
 *                       candidate list returned by listCanditate, rad.cpp:387)
 *   RAD_TIMES=path      one omp_get_wtime() stamp per step (step start)
 *   RAD_MAX_STEPS=k     stop after k shooter steps (as if converged)
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>
#include "rad.h"

extern "C" { long long rad_cnt[5]; }

namespace {
FILE *g_trace = nullptr;
long g_max_steps = -1;
long g_steps = 0;
std::vector<double> g_stamps;
bool g_init = false;

void init_once() {
    if (g_init) return;
    g_init = true;
    if (const char *p = getenv("RAD_TRACE")) g_trace = fopen(p, "w");
    if (const char *p = getenv("RAD_MAX_STEPS")) g_max_steps = atol(p);
}

template <typename T> void put(FILE *f, const T &v) { fwrite(&v, sizeof(T), 1, f); }

void at_exit_dump() {
    if (g_trace) { fclose(g_trace); g_trace = nullptr; }
    if (const char *p = getenv("RAD_TIMES")) {
        if (FILE *f = fopen(p, "w")) {
            for (double t : g_stamps) fprintf(f, "%.9f\n", t);
            fclose(f);
        }
    }
#ifdef RAD_COUNTERS
    fprintf(stderr, "[COUNT] rays %lld cells %lld tri_tests %lld se_tests %lld prec %lld\n",
            rad_cnt[0], rad_cnt[1], rad_cnt[2], rad_cnt[3], rad_cnt[4]);
#endif
    const char *path = getenv("RAD_DUMP");
    if (!path) return;
    FILE *f = fopen(path, "wb");
    if (!f) return;
    fwrite("RADDUMP1", 1, 8, f);
    int n = trinum;
    int esz = (int)sizeof(TriStore[0].area);
    int steps = (int)g_steps;
    put(f, n); put(f, esz); put(f, steps);
    /* field-major so the reader can map each array directly */
    for (int i = 0; i < n; i++) put(f, TriStore[i].parent);
    for (int i = 0; i < n; i++) for (int v = 0; v < 3; v++) for (int k = 0; k < 3; k++) put(f, TriStore[i].p[v][k]);
    for (int i = 0; i < n; i++) for (int v = 0; v < 3; v++) for (int k = 0; k < 3; k++) put(f, TriStore[i].accB[v][k]);
    for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) put(f, TriStore[i].deltaB[k]);
    for (int i = 0; i < n; i++) put(f, TriStore[i].area);
    for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) put(f, TriStore[i].n[k]);
    for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) put(f, TriStore[i].c[k]);
    for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) put(f, TriStore[i].Frgb[k]);
    for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) put(f, TriStore[i].neighbor[k]);
    fclose(f);
}

__attribute__((constructor)) void register_dump() { atexit(at_exit_dump); }
}  // namespace

bool rad_hook_shot(const std::vector<int> &C) {
    init_once();
    g_stamps.push_back(omp_get_wtime());
    if (g_max_steps >= 0 && g_steps >= g_max_steps) return true;
    if (g_trace) {
        fprintf(g_trace, "%zu", C.size());
        for (int c : C) fprintf(g_trace, " %d", c);
        fputc('\n', g_trace);
    }
    if (!C.empty()) g_steps++;
    return false;
}
