// ref_harness.cpp -- builds the reference's OWN CPU irregular-reduction code
// from its sources (never copied: the recipe in oracle/Makefile points the
// include path at the reference tree) and exposes it to the tests.
//
// TEST INFRASTRUCTURE ONLY.  Built into oracle/_ref/ (git-ignored), used by
// tests/ and tests/golden/make_golden.py in a container that holds the
// reference sources, to pin the oracle restatement (irr_oracle.c).
//
// Compiled twice:
//   -DREF_MOLDYN -I<ref>/moldyn : user function `map`  (moldyn/irregular.h:26-107)
//                                 executor compute_cpu (moldyn/irregular/cpu_kernel.cu:13-70)
//   -DREF_MINIMD -I<ref>/miniMD : user function `map1` (miniMD/irregular.h:109-163)
//
// The GPU half and the MPI half of the reference cannot build here (sm_20,
// CUDA 5.0 include path, no mpi.h); its CPU half needs only an empty
// __device__ and a member-initialising IrregularRuntime constructor, whose
// real definition (moldyn/irregular/irregular_runtime.cu:17-48) lives in a
// file that includes <mpi.h>.
#define __device__
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "lib/common.h"
#include "irregular/cpu_kernel.cu"
#include "irregular/cpu_kernel_tools.cu"

IrregularRuntime::IrregularRuntime(IRIndex ne, IRIndex nn, EDGE *e, void *ed, void *nd, int a,
                                   int b, int c, int d, void *co, int cs, void *p, int ps,
                                   int np, int ni)
    : global_num_edges_(ne), global_num_nodes_(nn), global_edges_(e), global_edge_data_(ed),
      global_node_data_(nd), edge_data_elm_size_(a), node_data_elm_size_(b),
      reduction_elm_size_(c), node_num_dims_(d), node_coordinates_(co), coordinate_size_(cs),
      parameter_size_(ps), parameter_(p), num_procs_(np), current_iter_(0), num_iters_(ni)
{
}

IrregularRuntime::~IrregularRuntime() {}

static void clear_object(Cobject *o)
{
    for (int b = 0; b < NUM_BUCKETS_G; b++) {
        o->keys[b] = EMPTY_BUCKET_VALUE;
        o->locks[b] = 0;
        o->pairs_per_bucket[b] = 0;
    }
}

extern "C" int ref_num_buckets(void) { return NUM_BUCKETS_G; }

// Runs the reference's map over every edge, serially, into one Cobject, the
// way one compute_cpu worker would with part_index all 0 and part_id 0.
// point_data is the reference's node layout (double xyz per node).
extern "C" int ref_map_all(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                           const void *param, float *out)
{
    if (n < 0 || n >= NUM_BUCKETS_G) return -1;
    Cobject *o = (Cobject *)malloc(sizeof(Cobject));
    int *part_index = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
    if (!o || !part_index) {
        free(o);
        free(part_index);
        return -1;
    }
    clear_object(o);
    FCPU::irmap_fp map_ptr = FCPU::map_function_table[0];
    FCPU::irreduce_fp reduce_ptr = FCPU::reduce_function_table[0];
    for (int64_t t = 0; t < e; t++)
        map_ptr(o, (void *)pos, part_index, (void *)edges, (void *)param, (unsigned)t, 0,
                reduce_ptr);
    for (int64_t k = 0; k < n; k++) {
        // hash(key) = key (irregular/hash.h:13-16): node k lives in bucket k
        int hit = o->keys[k] == (int)k;
        out[3 * k] = hit ? o->values[k].x : 0.0f;
        out[3 * k + 1] = hit ? o->values[k].y : 0.0f;
        out[3 * k + 2] = hit ? o->values[k].z : 0.0f;
    }
    free(o);
    free(part_index);
    return 0;
}

// Runs the reference's pthread executor compute_cpu with `threads` workers,
// as IrregularRuntime::launch does (moldyn/irregular/irregular_runtime.cu:
// 274-309), and merges the per-thread Cobjects into out (the reference's own
// merge_cobjects is broken, irregular_runtime.cu:413-434).  *seconds gets the
// fork-to-join wall time.
extern "C" int ref_compute_cpu(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                               const void *param, int param_size, int threads, float *out,
                               double *seconds)
{
    if (n < 0 || n >= NUM_BUCKETS_G || threads < 1 || e > 0x7fffffffLL) return -1;
    IrregularRuntime rt(e, n, (EDGE *)edges, NULL, (void *)pos, 0, 24, 24, 3, (void *)pos, 8,
                        (void *)param, param_size, 1, 1);
    // ~partition() frees its edge array (moldyn/irregular/partition.h:59-65), as the
    // reference hands it partitioner-owned copies: give it a private copy too.
    EDGE *edge_copy = (EDGE *)malloc(sizeof(EDGE) * (size_t)(e > 0 ? e : 1));
    if (!edge_copy) return -1;
    memcpy(edge_copy, edges, sizeof(EDGE) * (size_t)e);
    rt.p_cpu_ = new partition_cpu(n, (void *)pos, e, edge_copy, NULL, 24, 0, 24, 0, NULL);
    rt.part_index = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
    rt.roc_ = (Cobject *)malloc(sizeof(Cobject) * (size_t)threads);
    rt.cpu_edge_offset_ = (int *)malloc(sizeof(int));
    if (!rt.part_index || !rt.roc_ || !rt.cpu_edge_offset_) return -1;
    for (int t = 0; t < threads; t++) clear_object(&rt.roc_[t]);
    *rt.cpu_edge_offset_ = 0;
    rt.map_idx_ = 0;
    rt.reduce_idx_ = 0;
    pthread_mutex_t mutex;
    pthread_mutex_init(&mutex, NULL);
    CpuArgs *args = new CpuArgs[threads];
    pthread_t *tid = new pthread_t[threads];
    timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int t = 0; t < threads; t++) {
        args[t].tid = t;
        args[t].runtime = &rt;
        args[t].mutex = &mutex;
        pthread_create(&tid[t], NULL, compute_cpu, &args[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (seconds) *seconds = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    memset(out, 0, sizeof(float) * 3 * (size_t)n);
    for (int t = 0; t < threads; t++)
        for (int64_t k = 0; k < n; k++)
            if (rt.roc_[t].keys[k] == (int)k) {
                out[3 * k] += rt.roc_[t].values[k].x;
                out[3 * k + 1] += rt.roc_[t].values[k].y;
                out[3 * k + 2] += rt.roc_[t].values[k].z;
            }
    delete[] args;
    delete[] tid;
    delete rt.p_cpu_;
    rt.p_cpu_ = NULL;
    free(rt.part_index);
    free(rt.roc_);
    free(rt.cpu_edge_offset_);
    pthread_mutex_destroy(&mutex);
    return 0;
}
