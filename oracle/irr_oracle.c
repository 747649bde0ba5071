/*
 * irr_oracle.c -- CPU oracle for the irregular-reduction hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the reference results that tests/ and
 * __graft_entry__.smoke() compare against, and the timed CPU baseline of
 * bench.py.  The product library never links or
 * calls it.  Compile with -ffp-contract=off: every double and float operation
 * below is meant to round on its own, as the reference's CPU code does when
 * built without FMA contraction.
 *
 * Function-by-function provenance is in irr_oracle.h.
 */
#include "irr_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------ */
/* Per-edge law (FP64), as the reference's user functions evaluate it.       */
/* ------------------------------------------------------------------------ */

/* Minimum image of one coordinate difference: moldyn/irregular.h:51-60
 * applies `< -half -> += side` and then `> half -> -= side`. */
static inline double min_image(double d, double side, double half)
{
    if (d < -half) d += side;
    if (d > half) d -= side;
    return d;
}

/* Evaluates the law for edge (i, j).  Returns 1 when rd < cutoff2 and writes
 * d (the i - j separation) and the scalar s such that the force on i is d*s.
 * With periodic boundaries the scalar follows moldyn's chain
 * (moldyn/irregular.h:66-72: rrd7 - 0.5*rrd4); without, miniMD's
 * (miniMD/irregular.h:135-139: rrd3*(rrd3-0.5)*rrd). */
static inline int lj_edge_f64(const double *pos, int32_t i, int32_t j, const orc_lj_param *p,
                              double d[3], double *s, double *sabs_scalar)
{
    double xx = pos[3 * (int64_t)i] - pos[3 * (int64_t)j];
    double yy = pos[3 * (int64_t)i + 1] - pos[3 * (int64_t)j + 1];
    double zz = pos[3 * (int64_t)i + 2] - pos[3 * (int64_t)j + 2];
    if (p->periodic) {
        double half = 0.5 * p->side;
        xx = min_image(xx, p->side, half);
        yy = min_image(yy, p->side, half);
        zz = min_image(zz, p->side, half);
    }
    double rd = xx * xx + yy * yy + zz * zz;
    d[0] = xx;
    d[1] = yy;
    d[2] = zz;
    if (!(rd < p->cutoff2)) return 0;
    double rrd = 1.0 / rd;
    if (p->periodic) {
        double rrd2 = rrd * rrd;
        double rrd4 = rrd2 * rrd2;
        double rrd6 = rrd2 * rrd4;
        double rrd7 = rrd6 * rrd;
        *s = rrd7 - 0.5 * rrd4;
        if (sabs_scalar) *sabs_scalar = rrd7 + 0.5 * rrd4;
    } else {
        double rrd2 = rrd * rrd;
        double rrd3 = rrd2 * rrd;
        *s = rrd3 * (rrd3 - 0.5) * rrd;
        if (sabs_scalar) *sabs_scalar = rrd3 * (rrd3 + 0.5) * rrd;
    }
    return 1;
}

void orc_lj_reduce_f64(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                       const orc_lj_param *p, double *f, double *sabs)
{
    memset(f, 0, sizeof(double) * 3 * (size_t)n);
    if (sabs) memset(sabs, 0, sizeof(double) * 3 * (size_t)n);
    for (int64_t t = 0; t < e; t++) {
        int32_t i = edges[2 * t], j = edges[2 * t + 1];
        double d[3], s, sa;
        if (!lj_edge_f64(pos, i, j, p, d, &s, &sa)) continue;
        for (int c = 0; c < 3; c++) {
            double fc = d[c] * s;
            f[3 * (int64_t)i + c] += fc;
            f[3 * (int64_t)j + c] -= fc;
            if (sabs) {
                double a = fabs(d[c]) * sa;
                sabs[3 * (int64_t)i + c] += a;
                sabs[3 * (int64_t)j + c] += a;
            }
        }
    }
}

/* The scale of the per-result error metric: per node, the sum over its
 * in-cutoff edges of the FP64 edge force's largest component |f_e|inf. */
void orc_lj_edge_scale_inf(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                           const orc_lj_param *p, double *sinf)
{
    memset(sinf, 0, sizeof(double) * (size_t)n);
    for (int64_t t = 0; t < e; t++) {
        int32_t i = edges[2 * t], j = edges[2 * t + 1];
        double d[3], s;
        if (!lj_edge_f64(pos, i, j, p, d, &s, NULL)) continue;
        double m = 0.0;
        for (int c = 0; c < 3; c++) {
            const double a = fabs(d[c] * s);
            if (a > m) m = a;
        }
        sinf[i] += m;
        sinf[j] += m;
    }
}

void orc_lj_reduce_refnum_f32(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                              const orc_lj_param *p, float *f)
{
    memset(f, 0, sizeof(float) * 3 * (size_t)n);
    for (int64_t t = 0; t < e; t++) {
        int32_t i = edges[2 * t], j = edges[2 * t + 1];
        double d[3], s;
        if (!lj_edge_f64(pos, i, j, p, d, &s, NULL)) continue;
        /* VALUE forces = {xx*r148, ...} (float), insert(i, +forces), then
         * forces = -forces, insert(j, forces): moldyn/irregular.h:74-92. */
        float fx = (float)(d[0] * s), fy = (float)(d[1] * s), fz = (float)(d[2] * s);
        f[3 * (int64_t)i] += fx;
        f[3 * (int64_t)i + 1] += fy;
        f[3 * (int64_t)i + 2] += fz;
        f[3 * (int64_t)j] += -fx;
        f[3 * (int64_t)j + 1] += -fy;
        f[3 * (int64_t)j + 2] += -fz;
    }
}

/* ------------------------------------------------------------------------ */
/* CPU executor port (the timed CPU baseline).                               */
/* ------------------------------------------------------------------------ */

/* One worker's open-addressing table: identity hash, linear probing, one CAS
 * spin lock per bucket, float3 values.  Same shape as the reference's
 * Cobject (moldyn/irregular/roc.h:11-27) sized to n+1 buckets. */
typedef struct {
    int32_t *keys;
    float *vals;
    int32_t *locks;
} orc_table;

struct orc_exec {
    int64_t n;
    int64_t nb;
    int threads;
    orc_table *tab;
};

static void table_clear(orc_table *t, int64_t nb)
{
    for (int64_t b = 0; b < nb; b++) t->keys[b] = -1;
    memset(t->locks, 0, sizeof(int32_t) * (size_t)nb);
}

static inline void table_insert(orc_table *t, int64_t nb, int32_t key, const float v[3])
{
    int64_t b = (int64_t)((uint32_t)key % (uint64_t)nb);
    for (;;) {
        int32_t expect = 0;
        while (!__atomic_compare_exchange_n(&t->locks[b], &expect, 1, 0, __ATOMIC_ACQUIRE,
                                            __ATOMIC_RELAXED))
            expect = 0;
        if (t->keys[b] == -1) {
            t->keys[b] = key;
            t->vals[3 * b] = v[0];
            t->vals[3 * b + 1] = v[1];
            t->vals[3 * b + 2] = v[2];
            __atomic_store_n(&t->locks[b], 0, __ATOMIC_RELEASE);
            return;
        }
        if (t->keys[b] == key) {
            t->vals[3 * b] += v[0];
            t->vals[3 * b + 1] += v[1];
            t->vals[3 * b + 2] += v[2];
            __atomic_store_n(&t->locks[b], 0, __ATOMIC_RELEASE);
            return;
        }
        __atomic_store_n(&t->locks[b], 0, __ATOMIC_RELEASE);
        b = (b + 1) % nb;
    }
}

orc_exec *orc_exec_create(int64_t n, int threads)
{
    if (n < 0 || threads < 1) return NULL;
    orc_exec *x = (orc_exec *)calloc(1, sizeof(orc_exec));
    if (!x) return NULL;
    x->n = n;
    x->nb = n + 1;
    x->threads = threads;
    x->tab = (orc_table *)calloc((size_t)threads, sizeof(orc_table));
    if (!x->tab) {
        free(x);
        return NULL;
    }
    for (int t = 0; t < threads; t++) {
        x->tab[t].keys = (int32_t *)malloc(sizeof(int32_t) * (size_t)x->nb);
        x->tab[t].vals = (float *)malloc(sizeof(float) * 3 * (size_t)x->nb);
        x->tab[t].locks = (int32_t *)malloc(sizeof(int32_t) * (size_t)x->nb);
        if (!x->tab[t].keys || !x->tab[t].vals || !x->tab[t].locks) {
            orc_exec_destroy(x);
            return NULL;
        }
    }
    return x;
}

void orc_exec_destroy(orc_exec *x)
{
    if (!x) return;
    if (x->tab) {
        for (int t = 0; t < x->threads; t++) {
            free(x->tab[t].keys);
            free(x->tab[t].vals);
            free(x->tab[t].locks);
        }
        free(x->tab);
    }
    free(x);
}

typedef struct {
    orc_exec *x;
    int tid;
    const double *pos;
    int64_t e;
    const int32_t *edges;
    const orc_lj_param *p;
    int64_t chunk;
    int64_t *cursor;
    pthread_mutex_t *mutex;
} worker_arg;

/* The worker loop of compute_cpu (moldyn/irregular/cpu_kernel.cu:45-67):
 * grab `chunk` edges under the mutex, run the law on each, insert both
 * endpoint contributions into the private table. */
static void *worker(void *argp)
{
    worker_arg *a = (worker_arg *)argp;
    orc_table *tab = &a->x->tab[a->tid];
    int64_t nb = a->x->nb;
    for (;;) {
        pthread_mutex_lock(a->mutex);
        int64_t start = *a->cursor;
        *a->cursor += a->chunk;
        pthread_mutex_unlock(a->mutex);
        if (start >= a->e) break;
        int64_t end = start + a->chunk < a->e ? start + a->chunk : a->e;
        for (int64_t t = start; t < end; t++) {
            int32_t i = a->edges[2 * t], j = a->edges[2 * t + 1];
            double d[3], s;
            if (!lj_edge_f64(a->pos, i, j, a->p, d, &s, NULL)) continue;
            float v[3] = {(float)(d[0] * s), (float)(d[1] * s), (float)(d[2] * s)};
            table_insert(tab, nb, i, v);
            v[0] = -v[0];
            v[1] = -v[1];
            v[2] = -v[2];
            table_insert(tab, nb, j, v);
        }
    }
    return NULL;
}

static double now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
    orc_table *t;
    int64_t nb;
} clear_arg;

static void *clear_worker(void *argp)
{
    clear_arg *a = (clear_arg *)argp;
    table_clear(a->t, a->nb);
    return NULL;
}

/* Re-initialises every worker's table in parallel, one thread per table, as
 * re_init does (moldyn/irregular/irregular_runtime.cu:474-490). */
static void clear_tables(orc_exec *x)
{
    pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)x->threads);
    clear_arg *args = (clear_arg *)malloc(sizeof(clear_arg) * (size_t)x->threads);
    if (!tids || !args) {
        for (int t = 0; t < x->threads; t++) table_clear(&x->tab[t], x->nb);
    } else {
        for (int t = 0; t < x->threads; t++) {
            args[t].t = &x->tab[t];
            args[t].nb = x->nb;
            pthread_create(&tids[t], NULL, clear_worker, &args[t]);
        }
        for (int t = 0; t < x->threads; t++) pthread_join(tids[t], NULL);
    }
    free(tids);
    free(args);
}

static double exec_run_dpos(orc_exec *x, const double *pos, int64_t e, const int32_t *edges,
                            const orc_lj_param *p, int64_t chunk, float *f_out)
{
    if (!x || chunk < 1) return -1.0;
    clear_tables(x);
    pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)x->threads);
    worker_arg *args = (worker_arg *)malloc(sizeof(worker_arg) * (size_t)x->threads);
    if (!tids || !args) {
        free(tids);
        free(args);
        return -1.0;
    }
    pthread_mutex_t mutex;
    pthread_mutex_init(&mutex, NULL);
    int64_t cursor = 0;
    double t0 = now_seconds();
    for (int t = 0; t < x->threads; t++) {
        args[t] = (worker_arg){x, t, pos, e, edges, p, chunk, &cursor, &mutex};
        pthread_create(&tids[t], NULL, worker, &args[t]);
    }
    for (int t = 0; t < x->threads; t++) pthread_join(tids[t], NULL);
    double secs = now_seconds() - t0;
    pthread_mutex_destroy(&mutex);
    free(tids);
    free(args);
    if (f_out) {
        memset(f_out, 0, sizeof(float) * 3 * (size_t)x->n);
        for (int t = 0; t < x->threads; t++) {
            orc_table *tab = &x->tab[t];
            for (int64_t b = 0; b < x->nb; b++) {
                int32_t k = tab->keys[b];
                if (k < 0 || k >= x->n) continue;
                f_out[3 * (int64_t)k] += tab->vals[3 * b];
                f_out[3 * (int64_t)k + 1] += tab->vals[3 * b + 1];
                f_out[3 * (int64_t)k + 2] += tab->vals[3 * b + 2];
            }
        }
    }
    return secs;
}

double orc_exec_run(orc_exec *x, const float *pos, int64_t e, const int32_t *edges,
                    const orc_lj_param *p, int64_t chunk, float *f_out)
{
    /* The reference's node data is double xyz (moldyn/moldyn.h:32-37,
     * miniMD/ljs.cu:120-121): widen once, outside the timed region. */
    if (!x) return -1.0;
    double *dpos = (double *)malloc(sizeof(double) * 3 * (size_t)(x->n > 0 ? x->n : 1));
    if (!dpos) return -1.0;
    for (int64_t k = 0; k < 3 * x->n; k++) dpos[k] = (double)pos[k];
    double s = exec_run_dpos(x, dpos, e, edges, p, chunk, f_out);
    free(dpos);
    return s;
}

int orc_cpu_executor(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                     const orc_lj_param *p, int threads, int64_t chunk, float *f,
                     double *seconds)
{
    orc_exec *x = orc_exec_create(n, threads);
    if (!x) return -1;
    double s = exec_run_dpos(x, pos, e, edges, p, chunk, f);
    orc_exec_destroy(x);
    if (s < 0) return -1;
    if (seconds) *seconds = s;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Neighbour lists.                                                          */
/* ------------------------------------------------------------------------ */

/* The list criterion shared with the GPU builder, bit for bit. */
static inline int list_pair(const float *pos, int64_t i, int64_t j, float box, float hb,
                            float cut2)
{
    float d[3];
    for (int c = 0; c < 3; c++) {
        float v = pos[3 * i + c] - pos[3 * j + c];
        if (box > 0.0f) {
            if (v > hb)
                v = v - box;
            else if (v < -hb)
                v = v + box;
        }
        d[c] = v;
    }
    float a = d[0] * d[0];
    float b = d[1] * d[1];
    float r2 = a + b;
    float cz = d[2] * d[2];
    r2 = r2 + cz;
    return r2 <= cut2;
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

int64_t orc_neighbor_half_list(int64_t n, const float *pos, float box, float list_cut2,
                               int32_t *out, int64_t cap)
{
    return orc_neighbor_half_list_rows(n, pos, box, list_cut2, 0, n, out, cap);
}

int64_t orc_neighbor_half_list_rows(int64_t n, const float *pos, float box, float list_cut2,
                                    int64_t row_begin, int64_t row_end, int32_t *out, int64_t cap)
{
    if (n < 0 || list_cut2 < 0.0f || box < 0.0f) return -1;
    if (row_begin < 0) row_begin = 0;
    if (row_end > n) row_end = n;
    if (n == 0) return 0;
    float hb = 0.5f * box;
    float lo[3], hi[3];
    for (int c = 0; c < 3; c++) {
        lo[c] = pos[c];
        hi[c] = pos[c];
    }
    for (int64_t i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            if (pos[3 * i + c] < lo[c]) lo[c] = pos[3 * i + c];
            if (pos[3 * i + c] > hi[c]) hi[c] = pos[3 * i + c];
        }
    /* Cells at least slightly wider than the cutoff: pairs in range are in the
     * same or adjacent cells.  Periodic grids need >= 3 cells per axis so the
     * 27-cell neighbourhood visits each cell once; otherwise fall back to one
     * cell (all pairs). */
    double cut = sqrt((double)list_cut2) * 1.0001 + 1e-12;
    int nc[3];
    double org[3], csz[3];
    for (int c = 0; c < 3; c++) {
        double ext = box > 0.0f ? (double)box : (double)hi[c] - (double)lo[c];
        org[c] = box > 0.0f ? 0.0 : (double)lo[c];
        int k = (int)floor(ext / cut);
        if (box > 0.0f && k < 3) k = 1;
        if (k < 1) k = 1;
        if (k > 1024) k = 1024;
        nc[c] = k;
        csz[c] = ext > 0 ? ext / k : 1.0;
    }
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    int64_t *cell_of = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int64_t *start = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
    int32_t *sorted = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *row = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    if (!cell_of || !start || !sorted || !row) {
        free(cell_of);
        free(start);
        free(sorted);
        free(row);
        return -1;
    }
    for (int64_t i = 0; i < n; i++) {
        int64_t id[3];
        for (int c = 0; c < 3; c++) {
            int64_t k = (int64_t)floor(((double)pos[3 * i + c] - org[c]) / csz[c]);
            if (box > 0.0f) k = ((k % nc[c]) + nc[c]) % nc[c];
            if (k < 0) k = 0;
            if (k >= nc[c]) k = nc[c] - 1;
            id[c] = k;
        }
        cell_of[i] = (id[2] * nc[1] + id[1]) * nc[0] + id[0];
        start[cell_of[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; c++) start[c + 1] += start[c];
    {
        int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)ncell);
        memcpy(fill, start, sizeof(int64_t) * (size_t)ncell);
        for (int64_t i = 0; i < n; i++) sorted[fill[cell_of[i]]++] = (int32_t)i;
        free(fill);
    }
    int64_t count = 0;
    for (int64_t i = row_begin; i < row_end; i++) {
        int64_t c0 = cell_of[i];
        int64_t cx = c0 % nc[0], cy = (c0 / nc[0]) % nc[1], cz = c0 / ((int64_t)nc[0] * nc[1]);
        int64_t m = 0;
        /* distinct neighbour cells only (small grids revisit cells) */
        int64_t seen[27];
        int nseen = 0;
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int64_t x = cx + dx, y = cy + dy, z = cz + dz;
                    if (box > 0.0f) {
                        x = (x + nc[0]) % nc[0];
                        y = (y + nc[1]) % nc[1];
                        z = (z + nc[2]) % nc[2];
                    } else if (x < 0 || y < 0 || z < 0 || x >= nc[0] || y >= nc[1] || z >= nc[2]) {
                        continue;
                    }
                    int64_t cc = (z * nc[1] + y) * nc[0] + x;
                    int dup = 0;
                    for (int s = 0; s < nseen; s++) dup |= (seen[s] == cc);
                    if (dup) continue;
                    seen[nseen++] = cc;
                    for (int64_t q = start[cc]; q < start[cc + 1]; q++) {
                        int32_t j = sorted[q];
                        if (j <= i) continue;
                        if (list_pair(pos, i, j, box, hb, list_cut2)) row[m++] = j;
                    }
                }
        qsort(row, (size_t)m, sizeof(int32_t), cmp_i32);
        for (int64_t k = 0; k < m; k++) {
            if (out && count < cap) {
                out[2 * count] = (int32_t)i;
                out[2 * count + 1] = row[k];
            }
            count++;
        }
    }
    free(cell_of);
    free(start);
    free(sorted);
    free(row);
    return count;
}

void orc_fcc_moldyn(int m, double side, double *pos)
{
    /* moldyn/moldyn.cu:596-626: four interleaved simple-cubic sublattices,
     * node n, n+m^3, n+2m^3, n+3m^3. */
    int64_t np = (int64_t)m * m * m;
    double perturb = side / (double)m;
    for (int64_t n = 0; n < np; n++) {
        int64_t k = n % m;
        int64_t j = ((n - k) / m) % m;
        int64_t i = ((n - k - j * m) / ((int64_t)m * m)) % m;
        double *a = pos + 3 * n, *b = pos + 3 * (n + np), *c = pos + 3 * (n + 2 * np),
               *d = pos + 3 * (n + 3 * np);
        a[0] = i * perturb;
        a[1] = j * perturb;
        a[2] = k * perturb;
        b[0] = i * perturb + perturb * 0.5;
        b[1] = j * perturb + perturb * 0.5;
        b[2] = k * perturb;
        c[0] = i * perturb + perturb * 0.5;
        c[1] = j * perturb;
        c[2] = k * perturb + perturb * 0.5;
        d[0] = i * perturb;
        d[1] = j * perturb + perturb * 0.5;
        d[2] = k * perturb + perturb * 0.5;
    }
}

int64_t orc_fcc_minimd(int nx, int ny, int nz, double rho, double *pos, int64_t cap)
{
    /* miniMD/setup.cpp:44-57 (box) and :61-122 (lattice sites with
     * (i+j+k) even, half-lattice steps, kept when inside [0, prd)). */
    double alat = pow(4.0 / rho, 1.0 / 3.0);
    double xprd = nx * alat, yprd = ny * alat, zprd = nz * alat;
    int64_t cnt = 0;
    for (int k = 0; k <= 2 * nz - 1; k++)
        for (int j = 0; j <= 2 * ny - 1; j++)
            for (int i = 0; i <= 2 * nx - 1; i++) {
                if ((i + j + k) % 2 != 0) continue;
                double x = 0.5 * alat * i, y = 0.5 * alat * j, z = 0.5 * alat * k;
                if (x >= 0 && x < xprd && y >= 0 && y < yprd && z >= 0 && z < zprd) {
                    if (pos && cnt < cap) {
                        pos[3 * cnt] = x;
                        pos[3 * cnt + 1] = y;
                        pos[3 * cnt + 2] = z;
                    }
                    cnt++;
                }
            }
    return cnt;
}

/* ------------------------------------------------------------------------ */
/* Partition oracle.                                                         */
/* ------------------------------------------------------------------------ */

static inline uint32_t spread3(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

static inline uint32_t quant10(float x, float lo, float scale)
{
    float t = x - lo;
    t = t * scale;
    if (!(t > 0.0f)) return 0u;
    if (t >= 1023.0f) return 1023u;
    return (uint32_t)t;
}

void orc_morton_keys(int64_t n, const float *pos, const float lo[3], const float scale[3],
                     uint32_t *keys)
{
    for (int64_t i = 0; i < n; i++) {
        uint32_t qx = quant10(pos[3 * i], lo[0], scale[0]);
        uint32_t qy = quant10(pos[3 * i + 1], lo[1], scale[1]);
        uint32_t qz = quant10(pos[3 * i + 2], lo[2], scale[2]);
        keys[i] = spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
    }
}

/* Hilbert index of a cell on the 2^10-per-axis grid: Skilling's transform
 * (J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707, 2004)
 * from axes to the transposed index, whose bits are then interleaved with
 * axis 0 in the highest position of each 3-bit group. */
static uint32_t hilbert10(uint32_t x0, uint32_t x1, uint32_t x2)
{
    uint32_t X[3] = {x0, x1, x2};
    for (uint32_t Q = 1u << 9; Q > 1; Q >>= 1) {
        const uint32_t P = Q - 1;
        for (int i = 0; i < 3; i++) {
            if (X[i] & Q) {
                X[0] ^= P;  /* invert */
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;  /* exchange */
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0]; /* Gray encode */
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = 1u << 9; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    uint32_t key = 0;
    for (int b = 9; b >= 0; b--)
        key = (key << 3) | (((X[0] >> b) & 1u) << 2) | (((X[1] >> b) & 1u) << 1) | ((X[2] >> b) & 1u);
    return key;
}

void orc_hilbert_keys(int64_t n, const float *pos, const float lo[3], const float scale[3],
                      uint32_t *keys)
{
    for (int64_t i = 0; i < n; i++)
        keys[i] = hilbert10(quant10(pos[3 * i], lo[0], scale[0]), quant10(pos[3 * i + 1], lo[1], scale[1]),
                            quant10(pos[3 * i + 2], lo[2], scale[2]));
}

int orc_partition(int64_t n, const float *pos, const float lo[3], const float scale[3],
                  int64_t e, const int32_t *edges, int32_t *perm, int32_t *inv,
                  int64_t *row_off, int32_t *col)
{
    return orc_partition_curve(n, pos, lo, scale, 1, e, edges, perm, inv, row_off, col);
}

int orc_partition_curve(int64_t n, const float *pos, const float lo[3], const float scale[3],
                        int curve, int64_t e, const int32_t *edges, int32_t *perm, int32_t *inv,
                        int64_t *row_off, int32_t *col)
{
    if (n < 0 || e < 0) return -1;
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    if (!keys) return -1;
    if (curve == 0)
        orc_hilbert_keys(n, pos, lo, scale, keys);
    else
        orc_morton_keys(n, pos, lo, scale, keys);
    /* Stable counting sort on the 30-bit key, 3 passes of 10 bits. */
    int32_t *a = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t *b = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * 1025);
    if (!a || !b || !cnt) {
        free(keys);
        free(a);
        free(b);
        free(cnt);
        return -1;
    }
    for (int64_t i = 0; i < n; i++) a[i] = (int32_t)i;
    for (int pass = 0; pass < 3; pass++) {
        int sh = 10 * pass;
        memset(cnt, 0, sizeof(int64_t) * 1025);
        for (int64_t i = 0; i < n; i++) cnt[((keys[a[i]] >> sh) & 1023u) + 1]++;
        for (int d = 0; d < 1024; d++) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < n; i++) b[cnt[(keys[a[i]] >> sh) & 1023u]++] = a[i];
        int32_t *t = a;
        a = b;
        b = t;
    }
    for (int64_t i = 0; i < n; i++) {
        perm[i] = a[i];
        inv[a[i]] = (int32_t)i;
    }
    free(keys);
    free(a);
    free(b);
    free(cnt);
    /* Directed entries binned by row, stable in (edge, direction) order. */
    memset(row_off, 0, sizeof(int64_t) * (size_t)(n + 1));
    for (int64_t t = 0; t < e; t++) {
        int32_t i = edges[2 * t], j = edges[2 * t + 1];
        if (i < 0 || j < 0 || i >= n || j >= n) return -2;
        row_off[inv[i] + 1]++;
        row_off[inv[j] + 1]++;
    }
    for (int64_t r = 0; r < n; r++) row_off[r + 1] += row_off[r];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!fill) return -1;
    memcpy(fill, row_off, sizeof(int64_t) * (size_t)n);
    for (int64_t t = 0; t < e; t++) {
        int32_t ai = inv[edges[2 * t]], aj = inv[edges[2 * t + 1]];
        col[fill[ai]++] = aj;
        col[fill[aj]++] = ai;
    }
    free(fill);
    /* Columns of each row ascending: the canonical (row, col) order. */
    for (int64_t r = 0; r < n; r++)
        qsort(col + row_off[r], (size_t)(row_off[r + 1] - row_off[r]), sizeof(int32_t), cmp_i32);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Reference MD (FP64).                                                      */
/* ------------------------------------------------------------------------ */

static double wrap_box(double x, double L)
{
    x -= L * floor(x / L);
    if (x >= L) x -= L;
    if (x < 0.0) x = 0.0;
    return x;
}

/* The MD's work is split over `threads` host threads: the list by row ranges
 * (each range's pairs in the serial list's order, ranges concatenated in
 * order: the serial list exactly), the forces by edge ranges into per-thread
 * FP64 arrays summed in thread order (the FP64 result of another summation
 * order: ~1e-16 relative). */
typedef struct {
    int64_t n, r0, r1, cap, count;
    const float *fp;
    float box, cut2;
    int32_t *out;
} md_list_arg;

static void *md_list_worker(void *v)
{
    md_list_arg *a = (md_list_arg *)v;
    a->count = orc_neighbor_half_list_rows(a->n, a->fp, a->box, a->cut2, a->r0, a->r1, a->out, a->cap);
    return NULL;
}

static int64_t md_list(int64_t n, const double *pos, double side, double lc, float **fpos,
                       int32_t **edges, int threads)
{
    float *fp = *fpos;
    float Lf = (float)side;
    for (int64_t k = 0; k < 3 * n; k++) {
        float v = (float)pos[k];
        fp[k] = v >= Lf ? 0.0f : v;
    }
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    md_list_arg args[64];
    pthread_t tids[64];
    for (int t = 0; t < threads; t++) {
        md_list_arg a = {n, n * t / threads, n * (t + 1) / threads, 0, 0, fp, Lf, (float)(lc * lc), NULL};
        args[t] = a;
    }
    for (int t = 1; t < threads; t++) pthread_create(&tids[t], NULL, md_list_worker, &args[t]);
    md_list_worker(&args[0]);
    for (int t = 1; t < threads; t++) pthread_join(tids[t], NULL);
    int64_t e = 0;
    for (int t = 0; t < threads; t++) e += args[t].count;
    free(*edges);
    *edges = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)(e > 0 ? e : 1));
    int64_t off = 0;
    for (int t = 0; t < threads; t++) {
        args[t].out = *edges + 2 * off;
        args[t].cap = args[t].count;
        off += args[t].count;
    }
    for (int t = 1; t < threads; t++) pthread_create(&tids[t], NULL, md_list_worker, &args[t]);
    md_list_worker(&args[0]);
    for (int t = 1; t < threads; t++) pthread_join(tids[t], NULL);
    return e;
}

typedef struct {
    int64_t n, e0, e1;
    const double *pos;
    const int32_t *edges;
    const orc_lj_param *p;
    double *f;
    double u;
} md_force_arg;

static void *md_force_worker(void *v)
{
    md_force_arg *a = (md_force_arg *)v;
    double *f = a->f;
    memset(f, 0, sizeof(double) * 3 * (size_t)a->n);
    double u = 0.0;
    for (int64_t t = a->e0; t < a->e1; t++) {
        int32_t i = a->edges[2 * t], j = a->edges[2 * t + 1];
        double d[3], s;
        if (!lj_edge_f64(a->pos, i, j, a->p, d, &s, NULL)) continue;
        double rd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double r6 = 1.0 / (rd * rd * rd);
        u += 4.0 * r6 * (r6 - 1.0);
        for (int c = 0; c < 3; c++) {
            f[3 * (int64_t)i + c] += 48.0 * d[c] * s;
            f[3 * (int64_t)j + c] -= 48.0 * d[c] * s;
        }
    }
    a->u = u;
    return NULL;
}

/* part: threads - 1 scratch force arrays of 3n doubles (thread 0 writes f). */
static void md_forces(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                      const orc_lj_param *p, double *f, double *pe, int threads, double *part)
{
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    md_force_arg args[64];
    pthread_t tids[64];
    for (int t = 0; t < threads; t++) {
        md_force_arg a = {n, e * t / threads, e * (t + 1) / threads, pos, edges, p,
                          t == 0 ? f : part + (size_t)(t - 1) * 3 * (size_t)n, 0.0};
        args[t] = a;
    }
    for (int t = 1; t < threads; t++) pthread_create(&tids[t], NULL, md_force_worker, &args[t]);
    md_force_worker(&args[0]);
    for (int t = 1; t < threads; t++) pthread_join(tids[t], NULL);
    double u = args[0].u;
    for (int t = 1; t < threads; t++) {
        const double *g = args[t].f;
        for (int64_t k = 0; k < 3 * n; k++) f[k] += g[k];
        u += args[t].u;
    }
    if (pe) *pe = u;
}

/* The positions the forces are evaluated at: the FP64 state itself, or (as
 * the GPU evaluates them) its float copy, a value that rounds up to the box
 * side wrapping to 0, widened back to double. */
static const double *md_force_positions(int64_t n, const double *pos, double side, double *copy)
{
    if (!copy) return pos;
    const float Lf = (float)side;
    for (int64_t k = 0; k < 3 * n; k++) {
        const float v = (float)pos[k];
        copy[k] = (double)(v >= Lf ? 0.0f : v);
    }
    return copy;
}

int orc_md_run_mt(int64_t n, double *pos, double *vel, double side, double cutforce, double skin,
                  double dt, int steps, int rebuild_every, double *ke, double *pe, int threads,
                  int float_forces)
{
    if (n < 2 || !(side > 0) || rebuild_every < 1) return -1;
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    orc_lj_param p = {side, cutforce * cutforce, 1};
    float *fpos = (float *)malloc(sizeof(float) * 3 * (size_t)n);
    double *f = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *part = threads > 1 ? (double *)malloc(sizeof(double) * 3 * (size_t)n * (size_t)(threads - 1)) : NULL;
    double *copy = float_forces ? (double *)malloc(sizeof(double) * 3 * (size_t)n) : NULL;
    int32_t *edges = NULL;
    if (!fpos || !f || (threads > 1 && !part) || (float_forces && !copy)) {
        free(fpos);
        free(f);
        free(part);
        free(copy);
        return -1;
    }
    for (int64_t k = 0; k < 3 * n; k++) pos[k] = wrap_box(pos[k], side);
    int64_t e = md_list(n, pos, side, cutforce + skin, &fpos, &edges, threads);
    md_forces(n, md_force_positions(n, pos, side, copy), e, edges, &p, f, NULL, threads, part);
    int since = 0;
    for (int t = 0; t < steps; t++) {
        for (int64_t k = 0; k < 3 * n; k++) {
            vel[k] += 0.5 * dt * f[k];
            pos[k] = wrap_box(pos[k] + dt * vel[k], side);
        }
        if (++since >= rebuild_every) {
            e = md_list(n, pos, side, cutforce + skin, &fpos, &edges, threads);
            since = 0;
        }
        md_forces(n, md_force_positions(n, pos, side, copy), e, edges, &p, f, NULL, threads, part);
        for (int64_t k = 0; k < 3 * n; k++) vel[k] += 0.5 * dt * f[k];
    }
    if (pe) md_forces(n, md_force_positions(n, pos, side, copy), e, edges, &p, f, pe, threads, part);
    if (ke) {
        double s = 0.0;
        for (int64_t k = 0; k < 3 * n; k++) s += vel[k] * vel[k];
        *ke = 0.5 * s;
    }
    free(fpos);
    free(f);
    free(part);
    free(copy);
    free(edges);
    return 0;
}

int orc_md_run(int64_t n, double *pos, double *vel, double side, double cutforce, double skin,
               double dt, int steps, int rebuild_every, double *ke, double *pe)
{
    return orc_md_run_mt(n, pos, vel, side, cutforce, skin, dt, steps, rebuild_every, ke, pe, 1, 0);
}

/* ------------------------------------------------------------------------ */
/* Staged ("halo") layout (the library's own; see irr_oracle.h).             */
/* ------------------------------------------------------------------------ */

static int64_t staged_table(int64_t n, const int64_t *row_off, const int32_t *col, int64_t r0,
                            int64_t r1, int32_t *buf)
{
    int64_t m = 0;
    for (int64_t r = r0; r < r1 && r < n; r++) {
        buf[m++] = (int32_t)r;
        for (int64_t k = row_off[r]; k < row_off[r + 1]; k++) buf[m++] = col[k];
    }
    qsort(buf, (size_t)m, sizeof(int32_t), cmp_i32);
    int64_t u = 0;
    for (int64_t k = 0; k < m; k++)
        if (u == 0 || buf[u - 1] != buf[k]) buf[u++] = buf[k];
    return u;
}

static int64_t staged_slot(const int32_t *tab, int64_t ntab, int32_t id)
{
    int64_t lo = 0, hi = ntab;  /* first index with tab[idx] >= id */
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (tab[mid] < id) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

int orc_staged_layout(int64_t n, const int64_t *row_off, const int32_t *col, int slices_per_item,
                      int tab_max, int stream_max, int64_t *num_items, int64_t *num_words,
                      int64_t *num_ids, int32_t *items, uint32_t *slice_off, uint32_t *words,
                      int32_t *ids)
{
    if (n < 0 || slices_per_item < 1 || tab_max < 1 || stream_max < 64) return -2;
    const int64_t S = (n + 7) / 8;
    int64_t *cut = (int64_t *)malloc(sizeof(int64_t) * (size_t)(S + 1));  /* the cut's word counts */
    int64_t *soff = (int64_t *)malloc(sizeof(int64_t) * (size_t)(S + 1)); /* the slices' words */
    int64_t maxent = 0;
    for (int64_t r = 0; r < n; r++)
        if (row_off[r + 1] - row_off[r] > maxent) maxent = row_off[r + 1] - row_off[r];
    int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * (size_t)((int64_t)slices_per_item * 8 * (maxent + 1) + 8));
    uint16_t *rs = (uint16_t *)malloc(sizeof(uint16_t) * (size_t)(maxent + 1));
    int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(8 * slices_per_item));
    if (!cut || !soff || !buf || !rs || !order) {
        free(cut); free(soff); free(buf); free(rs); free(order);
        return -2;
    }
    int rc = 0;
    cut[0] = 0;
    for (int64_t q = 0; q < S && rc == 0; q++) {
        int64_t T = 0;
        for (int64_t r = 8 * q; r < 8 * q + 8 && r < n; r++) {
            int64_t t = (row_off[r + 1] - row_off[r] + 7) / 8;
            if (t > T) T = t;
        }
        if (32 * (T + 1) > stream_max) rc = -1;
        cut[q + 1] = cut[q] + 32 * (T + 1);
    }
    int64_t it = 0, tab0 = 0;
    int64_t q0 = 0;
    soff[0] = 0;
    while (q0 < S && rc == 0) {
        /* tentative run: at most slices_per_item blocks and stream_max words */
        int64_t q1 = q0 + 1;
        while (q1 < S && q1 - q0 < slices_per_item && cut[q1 + 1] - cut[q0] <= stream_max) q1++;
        /* cut into the longest prefixes whose tables fit */
        int64_t a = q0;
        while (a < q1 && rc == 0) {
            int64_t b = a + 1, ntab = staged_table(n, row_off, col, 8 * a, 8 * b, buf);
            if (ntab > tab_max) {
                rc = -1;
                break;
            }
            while (b < q1) {
                int64_t t2 = staged_table(n, row_off, col, 8 * a, 8 * (b + 1), buf);
                if (t2 > tab_max) break;
                b++;
            }
            ntab = staged_table(n, row_off, col, 8 * a, 8 * b, buf);
            const int64_t r0 = 8 * a, m = (8 * b < n ? 8 * b : n) - 8 * a, ns = b - a;
            /* the item's rows, longest first (ties by row id): insertion sort */
            for (int64_t k = 0; k < m; k++) {
                const int64_t r = r0 + k, len = row_off[r + 1] - row_off[r];
                int64_t pos = k;
                while (pos > 0) {
                    const int64_t o = order[pos - 1], lo = row_off[o + 1] - row_off[o];
                    if (lo >= len) break;
                    order[pos] = o;
                    pos--;
                }
                order[pos] = r;
            }
            for (int64_t j = 0; j < ns; j++) {
                int64_t T = 0;
                for (int64_t i = 8 * j; i < 8 * j + 8 && i < m; i++) {
                    const int64_t t = (row_off[order[i] + 1] - row_off[order[i]] + 7) / 8;
                    if (t > T) T = t;
                }
                soff[a + j + 1] = soff[a + j] + 32 * (T + 1);
            }
            if (items) {
                int32_t *w = items + 6 * it;
                w[0] = (int32_t)r0;
                w[1] = (int32_t)m;
                w[2] = (int32_t)soff[a];
                w[3] = (int32_t)(soff[b] - soff[a]);
                w[4] = (int32_t)tab0;
                w[5] = (int32_t)ntab;
            }
            if (ids) memcpy(ids + tab0, buf, sizeof(int32_t) * (size_t)ntab);
            if (words) {
                for (int64_t j = 0; j < ns; j++) {
                    const int64_t q = a + j;
                    const int64_t T = (soff[q + 1] - soff[q]) / 32 - 1;
                    uint32_t *sw = words + soff[q];
                    for (int i = 0; i < 8; i++) {
                        const int64_t pos = 8 * j + i;
                        int64_t len = 0, own = 0;
                        int64_t cnt[8] = {0}, cur[8] = {0}, beg[8] = {0};
                        uint32_t hdr = 1u << 31;  /* a padding row */
                        if (pos < m) {
                            const int64_t r = order[pos];
                            len = row_off[r + 1] - row_off[r];
                            own = staged_slot(buf, ntab, (int32_t)r);
                            hdr = (uint32_t)(own * 16) | ((uint32_t)len << 14) | ((uint32_t)(r - r0) << 24);
                            /* the row's slots bucketed by bank group, ascending */
                            for (int64_t k = 0; k < len; k++) cnt[staged_slot(buf, ntab, col[row_off[r] + k]) & 7]++;
                            int64_t acc = 0;
                            for (int g = 0; g < 8; g++) {
                                beg[g] = acc;
                                acc += cnt[g];
                            }
                            int64_t fill[8];
                            for (int g = 0; g < 8; g++) fill[g] = beg[g];
                            for (int64_t k = 0; k < len; k++) {
                                const int64_t sl = staged_slot(buf, ntab, col[row_off[r] + k]);
                                rs[fill[sl & 7]++] = (uint16_t)sl;
                            }
                        }
                        for (int l = 0; l < 4; l++) sw[4 * i + l] = hdr;
                        const int p = i & 1;
                        for (int64_t t = 0; t < T; t++) {
                            uint32_t pk[2][4];
                            for (int h = 0; h < 2; h++)
                                for (int l = 0; l < 4; l++) {
                                    int g = (int)((2 * t + h + 4 * p + l) & 7);
                                    if (cur[g] >= cnt[g]) {
                                        int best = -1;
                                        for (int x = 0; x < 8; x++)
                                            if (cnt[x] - cur[x] > 0 && (best < 0 || cnt[x] - cur[x] > cnt[best] - cur[best]))
                                                best = x;
                                        g = best;
                                    }
                                    int64_t slot = own;
                                    if (g >= 0) slot = rs[beg[g] + cur[g]++];
                                    pk[h][l] = (uint32_t)(slot * 16);
                                }
                            for (int l = 0; l < 4; l++)
                                sw[32 * (t + 1) + 4 * i + l] = pk[0][l] | (pk[1][l] << 16);
                        }
                    }
                }
            }
            it++;
            tab0 += ntab;
            a = b;
        }
        q0 = q1;
    }
    if (rc == 0) {
        if (slice_off)
            for (int64_t q = 0; q <= S; q++) slice_off[q] = (uint32_t)soff[q];
        if (num_items) *num_items = it;
        if (num_words) *num_words = soff[S];
        if (num_ids) *num_ids = tab0;
    }
    free(cut);
    free(soff);
    free(buf);
    free(rs);
    free(order);
    return rc;
}
