/*
 * Minimal stand-in for the hwloc API subset used by the reference's
 * solidfmm/multithreaded_translator.cpp (topology init/load/destroy, core
 * enumeration, cpuset dup/singlify/free, thread binding, membind).
 *
 * TEST INFRASTRUCTURE: only used to compile the reference library into
 * oracle/_ref/ as a checker and CPU baseline.  hwloc itself is not installed
 * on either machine.  "Cores" are the CPUs in the process affinity mask; a
 * cpuset is a single CPU id; binding uses pthread_setaffinity_np.
 */
#ifndef SFMM_ORACLE_HWLOC_SHIM_H
#define SFMM_ORACLE_HWLOC_SHIM_H

#ifndef _GNU_SOURCE
#define _GNU_SOURCE
#endif
#include <pthread.h>
#include <sched.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

struct hwloc_bitmap_s { int cpu; };
struct hwloc_obj_s { struct hwloc_bitmap_s *cpuset; };
struct hwloc_topology { int ncpu; int *cpus; struct hwloc_obj_s *objs; struct hwloc_bitmap_s *sets; };

typedef struct hwloc_topology *hwloc_topology_t;
typedef struct hwloc_bitmap_s *hwloc_cpuset_t;
typedef struct hwloc_bitmap_s *hwloc_bitmap_t;
typedef struct hwloc_obj_s *hwloc_obj_t;

typedef enum { HWLOC_OBJ_CORE = 5 } hwloc_obj_type_t;
enum { HWLOC_CPUBIND_THREAD = 1 << 1, HWLOC_CPUBIND_STRICT = 1 << 2 };
enum { HWLOC_MEMBIND_NEXTTOUCH = 4 };
enum { HWLOC_MEMBIND_THREAD = 1 << 1 };

static inline int hwloc_topology_init(hwloc_topology_t *t)
{
    *t = (hwloc_topology_t)calloc(1, sizeof(struct hwloc_topology));
    return *t ? 0 : -1;
}

static inline int hwloc_topology_load(hwloc_topology_t t)
{
    cpu_set_t mask;
    CPU_ZERO(&mask);
    if (sched_getaffinity(0, sizeof(mask), &mask) != 0) return -1;
    int n = CPU_COUNT(&mask);
    const char *lim = getenv("SFMM_REF_THREADS");
    int cap = lim ? atoi(lim) : 0;
    if (cap > 0 && cap < n) n = cap;
    t->cpus = (int *)calloc((size_t)n, sizeof(int));
    t->objs = (struct hwloc_obj_s *)calloc((size_t)n, sizeof(struct hwloc_obj_s));
    t->sets = (struct hwloc_bitmap_s *)calloc((size_t)n, sizeof(struct hwloc_bitmap_s));
    if (!t->cpus || !t->objs || !t->sets) return -1;
    int k = 0;
    for (int c = 0; c < CPU_SETSIZE && k < n; ++c)
        if (CPU_ISSET(c, &mask)) {
            t->cpus[k] = c;
            t->sets[k].cpu = c;
            t->objs[k].cpuset = &t->sets[k];
            ++k;
        }
    t->ncpu = k;
    return 0;
}

static inline void hwloc_topology_destroy(hwloc_topology_t t)
{
    if (!t) return;
    free(t->cpus);
    free(t->objs);
    free(t->sets);
    free(t);
}

static inline int hwloc_topology_abi_check(hwloc_topology_t t) { return t ? 0 : -1; }
static inline int hwloc_get_type_or_below_depth(hwloc_topology_t t, hwloc_obj_type_t ty)
{
    (void)t; (void)ty;
    return 0;
}
static inline int hwloc_get_nbobjs_by_depth(hwloc_topology_t t, int depth)
{
    (void)depth;
    return t->ncpu;
}
static inline hwloc_obj_t hwloc_get_obj_by_depth(hwloc_topology_t t, int depth, unsigned i)
{
    (void)depth;
    return &t->objs[i];
}
static inline hwloc_bitmap_t hwloc_bitmap_dup(const struct hwloc_bitmap_s *s)
{
    hwloc_bitmap_t b = (hwloc_bitmap_t)malloc(sizeof(struct hwloc_bitmap_s));
    if (b) *b = *s;
    return b;
}
static inline int hwloc_bitmap_singlify(hwloc_bitmap_t b)
{
    (void)b;
    return 0;
}
static inline void hwloc_bitmap_free(hwloc_bitmap_t b) { free(b); }
static inline int hwloc_set_cpubind(hwloc_topology_t t, const struct hwloc_bitmap_s *s, int flags)
{
    (void)t; (void)flags;
    cpu_set_t mask;
    CPU_ZERO(&mask);
    CPU_SET(s->cpu, &mask);
    return pthread_setaffinity_np(pthread_self(), sizeof(mask), &mask) ? -1 : 0;
}
static inline int hwloc_set_membind(hwloc_topology_t t, const struct hwloc_bitmap_s *s, int policy, int flags)
{
    (void)t; (void)s; (void)policy; (void)flags;
    return 0;
}

#ifdef __cplusplus
}
#endif
#endif
