// Stress check of the host thread pool behind the packing passes
// (split_range, for_each_item in csrc/prep_workspace.h): three threads run
// passes of random sizes and thread counts at the same time; every index must
// be visited exactly once per pass.  Built and run by tests/test_host_pool.py.
#include "prep_workspace.h"
#include <cstdio>
#include <vector>
using namespace radgb;
int main() {
    long bad = 0;
    auto worker = [&](int seed) {
        for (int it = 0; it < 20000; it++) {
            int n = 1000 + (it * 7919 + seed) % 50000;
            std::vector<int> v(n, 0);
            int jobs = 1 + (it + seed) % 16;
            if (it & 1) split_range(n, jobs, [&](int a, int b) { for (int i = a; i < b; i++) v[i] += i; });
            else for_each_item(n % 300 + 1, jobs, [&](int k) { v[k] += k; });
            int m = (it & 1) ? n : n % 300 + 1;
            for (int i = 0; i < m; i++) if (v[i] != i) { bad++; break; }
        }
    };
    std::thread a(worker, 1), b(worker, 2);
    worker(3);
    a.join(); b.join();
    printf("bad %ld\n", bad);
    return bad != 0;
}
