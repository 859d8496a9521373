/* Counter macros force-included into the staged reference build.
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 * With RAD_COUNTERS undefined every macro is empty, so the timed reference
 * binary runs the reference's code unchanged. */
#ifndef RAD_REF_HOOKS_H
#define RAD_REF_HOOKS_H
#ifdef RAD_COUNTERS
#ifdef __cplusplus
extern "C" {
#endif
extern long long rad_cnt[5];
#ifdef __cplusplus
}
#endif
#define RAD_CNT_RAY()  __atomic_fetch_add(&rad_cnt[0], 1, __ATOMIC_RELAXED)
#define RAD_CNT_CELL() __atomic_fetch_add(&rad_cnt[1], 1, __ATOMIC_RELAXED)
#define RAD_CNT_TRI()  __atomic_fetch_add(&rad_cnt[2], 1, __ATOMIC_RELAXED)
#define RAD_CNT_SE()   __atomic_fetch_add(&rad_cnt[3], 1, __ATOMIC_RELAXED)
#define RAD_CNT_PREC() __atomic_fetch_add(&rad_cnt[4], 1, __ATOMIC_RELAXED)
#else
#define RAD_CNT_RAY()
#define RAD_CNT_CELL()
#define RAD_CNT_TRI()
#define RAD_CNT_SE()
#define RAD_CNT_PREC()
#endif
#endif
