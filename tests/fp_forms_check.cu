// Checks the FP32 forms add_tenth and ff_scale (rad_kernels.cuh) against the
// double expressions they stand for, bit for bit.
//   fp_forms_check cpu STRIDE N   host: every STRIDE-th float bit pattern for
//                                 add_tenth, N random ff_scale triples
//   fp_forms_check gpu N          the same on the device (N inputs each)
// Prints "ok <cases> <fallbacks...>" or the first mismatch; exit status 1 on
// a mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>

#include "rad_kernels.cuh"

using radgb::dev::add_tenth;
using radgb::dev::ff_scale;
using radgb::dev::f2u;
using radgb::dev::u2f;

static __host__ __device__ inline float tenth_ref(float x) { return (float)((double)x + 0.1); }
static __host__ __device__ inline float scale_ref(float f, float a, float d2) {
    return (float)((double)f * ((double)a / ((double)d2 * radgb::dev::kPiD)));
}
static __host__ __device__ inline bool same(float a, float b) {
    return f2u(a) == f2u(b) || (a != a && b != b);
}

// splitmix64: a deterministic stream of test inputs
static __host__ __device__ inline unsigned long long mix(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
// log-uniform positive float with exponent in [lo, hi)
static __host__ __device__ inline float logu(unsigned long long r, int lo, int hi) {
    const unsigned e = (unsigned)(lo + (int)((r >> 40) % (unsigned)(hi - lo))) + 127u;
    return u2f((e << 23) | (unsigned)(r & 0x7fffffu));
}
// triple i: mostly the solver's ranges; every 8th is pushed next to a float
// rounding midpoint of the exact result, where the fallback must answer
static __host__ __device__ inline void triple(unsigned long long i, float& f, float& a, float& d2) {
    const unsigned long long r1 = mix(3 * i), r2 = mix(3 * i + 1), r3 = mix(3 * i + 2);
    f = logu(r1, -40, 1);
    a = logu(r2, -30, 20);
    d2 = logu(r3, -30, 30);
    if ((i & 7) == 0) {
        // choose d2 so that f*a/(d2*pi) is close to the midpoint y+spacing/2
        const double y = (double)scale_ref(f, a, d2);
        const double mid = y + (double)(u2f((f2u((float)y) & 0x7f800000u) - (23u << 23))) * 0.5;
        const double want = (double)f * (double)a / (mid * radgb::dev::kPiD);
        d2 = (float)want;
    }
}

__global__ void k_check(unsigned long long n, unsigned long long* bad, unsigned long long* first) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = u2f((unsigned)mix(i ^ 0x5555ull));
    if (!same(add_tenth(x), tenth_ref(x))) {
        atomicAdd(bad, 1ull);
        atomicMin(first, i);
    }
    float f, a, d2;
    triple(i, f, a, d2);
    if (!same(ff_scale(f, a, d2), scale_ref(f, a, d2))) {
        atomicAdd(bad + 1, 1ull);
        atomicMin(first + 1, i);
    }
}

int main(int argc, char** argv) {
    if (argc >= 2 && !strcmp(argv[1], "cpu")) {
        const unsigned long long stride = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
        const unsigned long long n = argc > 3 ? strtoull(argv[3], 0, 10) : 1000000;
        unsigned long long cases = 0;
        for (unsigned long long b = 0; b <= 0xffffffffull; b += stride) {
            const float x = u2f((unsigned)b);
            const float got = add_tenth(x), want = tenth_ref(x);
            if (!same(got, want)) {
                printf("add_tenth mismatch x=%a got=%a want=%a\n", x, got, want);
                return 1;
            }
            ++cases;
        }
        unsigned long long scases = 0;
        for (unsigned long long i = 0; i < n; i++) {
            float f, a, d2;
            triple(i, f, a, d2);
            const float got = ff_scale(f, a, d2), want = scale_ref(f, a, d2);
            if (!same(got, want)) {
                printf("ff_scale mismatch f=%a a=%a d2=%a got=%a want=%a\n", f, a, d2, got, want);
                return 1;
            }
            ++scases;
        }
        printf("ok %llu %llu\n", cases, scases);
        return 0;
    }
    if (argc >= 2 && !strcmp(argv[1], "gpu")) {
        const unsigned long long n = argc > 2 ? strtoull(argv[2], 0, 10) : 1 << 24;
        unsigned long long *d, h[4] = {0, 0, ~0ull, ~0ull};
        if (cudaMalloc(&d, sizeof h) != cudaSuccess) return 2;
        cudaMemcpy(d, h, sizeof h, cudaMemcpyHostToDevice);
        k_check<<<(unsigned)((n + 255) / 256), 256>>>(n, d, d + 2);
        if (cudaDeviceSynchronize() != cudaSuccess) { printf("cuda error\n"); return 2; }
        cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
        if (h[0] || h[1]) {
            printf("mismatch add_tenth %llu (first %llu) ff_scale %llu (first %llu)\n", h[0], h[2], h[1], h[3]);
            return 1;
        }
        printf("ok %llu\n", n);
        return 0;
    }
    fprintf(stderr, "usage: fp_forms_check cpu STRIDE N | gpu N\n");
    return 2;
}
