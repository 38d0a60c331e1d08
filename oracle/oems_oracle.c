/*
 * oems_oracle.c -- ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C CPU restatement of openEMS's EC-FDTD engine path, used by the tests (as the
 * checker of the CUDA engine), by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.
 * Nothing in the product imports, links or calls this file.
 *
 * It exposes the same C ABI shape as include/oems_cuda.h with the prefix oems_ref_ and two
 * storage modes:
 *
 *  - "basic": fields and coefficients in N-I-J-K order, updated exactly like Engine
 *    (FDTD/engine.cpp:110-222), one thread.  This is the semantic reference: separate float
 *    multiply and add (build with -ffp-contract=off), no flush-to-zero.
 *  - "mt":    the default openEMS engine, multithreaded SSE-compressed: fields as 4-lane
 *    vectors in I-J-K-N order (tools/arraylib/array_e.h:53-61) with lane-strided z
 *    (FDTD/engine_sse.h:38-47), coefficients deduplicated per 4-lane vector like
 *    Operator_SSE_Compressed::CompressOperator (FDTD/operator_sse_compressed.cpp:114-175), the
 *    update of Engine_SSE_Compressed (FDTD/engine_sse_compressed.cpp:51-311) and the x-slab
 *    thread driver of NS_Engine_Multithread::thread::operator() (FDTD/engine_multithread.cpp:
 *    310-402) with pthread barriers.  Its results equal the basic mode's bit for bit, which is
 *    the reference's own engine contract (TESTSUITE/enginetests/cavity.m).
 *
 * Extensions follow the reference's phase order and priorities (FDTD/engine.cpp:224-286,
 * FDTD/extensions/engine_extension.h:21-29): pre hooks in reverse priority, post/apply hooks in
 * priority order: UPML (+1e6), then Lorentz (0, inserted after Mur), Mur walls (0, reverse
 * insertion), excitation (-1000).
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#undef I /* complex.h's imaginary unit; this file names a current field I */

typedef float v4sf __attribute__((vector_size(16)));

#define OK 0
#define ERR_ARG 1
#define ERR_STATE 3
#define ERR_UNSUPPORTED 4
#define ERR_NOMEM 6

#define EPS0 8.85418781762e-12
#define MUE0 1.256637062e-6
#define M_PI_REF 3.14159265358979323846

#define MAX_UPML 6
#define MAX_MUR 6
#define MAX_LOR 16
#define MAX_PROBES 256
#define MAX_DUMPS 64

typedef struct {
    unsigned start[3], nl[3];
    size_t n;
    float *vv, *vvfo, *vvfn, *ii, *iifo, *iifn, *vflux, *iflux;
} upml_t;

typedef struct {
    int ny, nyP, nyPP;
    unsigned line, shift, start_ts, n1, n2;
    float *cP, *cPP, *bP, *bPP;
} mur_t;

typedef struct {
    unsigned count;
    unsigned *pos;
    int von, con, vlon, clon;
    float *vint, *vext, *vlor, *iint, *iext, *ilor;
    float *vade, *vlade, *iade, *ilade;
} lor_t;

typedef struct {
    int type; /* 0 voltage, 1 current, 2 E field, 3 H field */
    unsigned start[3], stop[3];
    double el[3]; /* field probes: edge length of each component at start (E main, H dual mesh) */
    unsigned ncomp; /* values per sample: 1, or 3 for a field probe */
    int nd, si[3], ei[3];
    double weight;
    unsigned interval, start_ts, stop_ts;
    double *series;
    size_t nslots;
    unsigned fd_interval, nf;
    double *freqs;
    double *dft;
} probe_t;

typedef struct {
    int field;
    int interp; /* 0 none, 1 node, 2 cell interpolation */
    /* time-domain dump: samples kept in memory, float [nsamp][3][sx][sy][sz] */
    int td;
    unsigned td_interval, td_start, td_stop, nsamp, cap;
    unsigned *samp_ts;
    float *samples;
    unsigned start[3], stop[3], sz[3];
    unsigned fd_interval, nf;
    double *freqs;
    double *el[3], *del[3];
    double *rho; /* cylindrical mesh: rho of each x line of the dump's mesh, else NULL */
    float *acc; /* [nf][3][sx][sy][sz][2] */
} dump_t;

typedef struct oems_ref_engine {
    unsigned N[3];
    size_t cells;
    double dt;
    unsigned numTS, maxTS;
    int inited;
    /* basic */
    float *volt, *curr;
    float *vv, *vi, *ii, *iv;
    /* mt */
    int mt, nthreads;
    unsigned nv;
    v4sf *f4volt, *f4curr;
    unsigned *op_index;
    unsigned nclasses;
    v4sf *cvv, *cvi, *cii, *civ; /* [3][nclasses] */
    pthread_t *threads;
    pthread_barrier_t bar_iter, bar_start, bar_stop;
    unsigned *tstart, *tstop, *tstop_h;
    volatile int stop_threads;
    unsigned iter_ts;
    /* excitation */
    unsigned nV, nI, sig_len, period;
    unsigned *v_idx, *i_idx, *v_delay, *i_delay;
    unsigned short *v_dir, *i_dir;
    float *v_amp, *i_amp, *sig_v, *sig_i;
    /* TFSF plane wave: terms in the reference's application order */
    unsigned tf_nV, tf_nI, tf_len, tf_period, tf_max_delay;
    unsigned *tf_v_idx, *tf_i_idx, *tf_v_delay, *tf_i_delay, *tf_lut;
    unsigned short *tf_v_dir, *tf_i_dir;
    float *tf_v_delta, *tf_i_delta, *tf_v_amp, *tf_i_amp, *tf_sig_v, *tf_sig_i;
    /* lumped RLC loads: coefficients and the reference's rotating state buffers */
    unsigned rlc_n;
    unsigned *rlc_pos;
    int *rlc_dir;
    float *rlc_c; /* [9][n]: ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2 */
    float *rlc_il, *rlc_vd[3], *rlc_j[3];
    /* Engine_Ext_Cylinder: closed alpha mesh, rho = 0 on it, the axis coefficients [Nz] */
    int cyl_closed, cyl_r0;
    float *cyl_vv_r0, *cyl_vi_r0;
    /* extensions */
    upml_t upml[MAX_UPML];
    int nupml;
    mur_t mur[MAX_MUR];
    int nmur;
    lor_t lor[MAX_LOR];
    int nlor;
    probe_t probes[MAX_PROBES];
    int nprobes;
    dump_t dumps[MAX_DUMPS];
    int ndumps;
    char err[512];
} eng_t;

/* ------------------------------------------------------------------------------------------ */
/* field access: Engine::GetVolt / Engine_sse::GetVolt (FDTD/engine.h:55-101, engine_sse.h:38-84) */

static inline size_t nijk(const eng_t *e, unsigned n, unsigned x, unsigned y, unsigned z)
{
    return (((size_t)n * e->N[0] + x) * e->N[1] + y) * e->N[2] + z;
}

static inline float *fptr(eng_t *e, int curr, unsigned n, unsigned x, unsigned y, unsigned z)
{
    if (!e->mt)
        return (curr ? e->curr : e->volt) + nijk(e, n, x, y, z);
    unsigned v = z % e->nv, l = z / e->nv;
    v4sf *base = curr ? e->f4curr : e->f4volt;
    return ((float *)&base[(((size_t)x * e->N[1] + y) * e->nv + v) * 3 + n]) + l;
}

#define GETV(e, n, x, y, z) (*fptr((e), 0, (n), (x), (y), (z)))
#define GETI(e, n, x, y, z) (*fptr((e), 1, (n), (x), (y), (z)))

static void *xcalloc(size_t n, size_t s)
{
    if (n == 0)
        n = 1;
    return calloc(n, s);
}

static float *dupf(const float *src, size_t n)
{
    if (!src)
        return NULL;
    float *d = (float *)xcalloc(n, sizeof(float));
    if (d)
        memcpy(d, src, n * sizeof(float));
    return d;
}

/* ------------------------------------------------------------------------------------------ */
/* lifecycle */

static int create_common(const unsigned nl[3], double dt, eng_t **out)
{
    if (!nl || !out || nl[0] < 2 || nl[1] < 2 || nl[2] < 2 || !(dt > 0))
        return ERR_ARG;
    eng_t *e = (eng_t *)calloc(1, sizeof(eng_t));
    if (!e)
        return ERR_NOMEM;
    memcpy(e->N, nl, sizeof(e->N));
    e->cells = (size_t)nl[0] * nl[1] * nl[2];
    e->dt = dt;
    *out = e;
    return OK;
}

int oems_ref_create(const unsigned nl[3], double dt, int device, eng_t **out)
{
    (void)device;
    int rc = create_common(nl, dt, out);
    if (rc)
        return rc;
    eng_t *e = *out;
    e->volt = (float *)xcalloc(3 * e->cells, sizeof(float));
    e->curr = (float *)xcalloc(3 * e->cells, sizeof(float));
    if (!e->volt || !e->curr)
        return ERR_NOMEM;
    return OK;
}

/* The multithreaded SSE-compressed engine (Engine_Multithread over Engine_SSE_Compressed). */
int oems_ref_create_mt(const unsigned nl[3], double dt, int nthreads, eng_t **out)
{
    int rc = create_common(nl, dt, out);
    if (rc)
        return rc;
    eng_t *e = *out;
    e->mt = 1;
    e->nthreads = nthreads > 0 ? nthreads : 1;
    e->nv = (unsigned)ceil((double)nl[2] / 4.0); /* FDTD/engine_sse.cpp:40 */
    size_t nvec = (size_t)nl[0] * nl[1] * e->nv * 3;
    e->f4volt = (v4sf *)aligned_alloc(16, nvec * sizeof(v4sf));
    e->f4curr = (v4sf *)aligned_alloc(16, nvec * sizeof(v4sf));
    if (!e->f4volt || !e->f4curr)
        return ERR_NOMEM;
    memset(e->f4volt, 0, nvec * sizeof(v4sf));
    memset(e->f4curr, 0, nvec * sizeof(v4sf));
    return OK;
}

static void stop_threads(eng_t *e);

void oems_ref_destroy(eng_t *e)
{
    if (!e)
        return;
    if (e->threads)
        stop_threads(e);
    free(e->volt); free(e->curr);
    free(e->vv); free(e->vi); free(e->ii); free(e->iv);
    free(e->f4volt); free(e->f4curr); free(e->op_index);
    free(e->cvv); free(e->cvi); free(e->cii); free(e->civ);
    free(e->tstart); free(e->tstop); free(e->tstop_h);
    free(e->v_idx); free(e->i_idx); free(e->v_delay); free(e->i_delay);
    free(e->v_dir); free(e->i_dir); free(e->v_amp); free(e->i_amp); free(e->sig_v); free(e->sig_i);
    free(e->tf_v_idx); free(e->tf_i_idx); free(e->tf_v_delay); free(e->tf_i_delay); free(e->tf_lut);
    free(e->tf_v_dir); free(e->tf_i_dir); free(e->tf_v_delta); free(e->tf_i_delta);
    free(e->tf_v_amp); free(e->tf_i_amp); free(e->tf_sig_v); free(e->tf_sig_i);
    free(e->cyl_vv_r0); free(e->cyl_vi_r0);
    free(e->rlc_pos); free(e->rlc_dir); free(e->rlc_c); free(e->rlc_il);
    for (int q = 0; q < 3; ++q) { free(e->rlc_vd[q]); free(e->rlc_j[q]); }
    for (int r = 0; r < e->nupml; ++r) {
        upml_t *u = &e->upml[r];
        free(u->vv); free(u->vvfo); free(u->vvfn); free(u->ii); free(u->iifo); free(u->iifn);
        free(u->vflux); free(u->iflux);
    }
    for (int w = 0; w < e->nmur; ++w) {
        mur_t *m = &e->mur[w];
        free(m->cP); free(m->cPP); free(m->bP); free(m->bPP);
    }
    for (int o = 0; o < e->nlor; ++o) {
        lor_t *l = &e->lor[o];
        free(l->pos); free(l->vint); free(l->vext); free(l->vlor); free(l->iint); free(l->iext); free(l->ilor);
        free(l->vade); free(l->vlade); free(l->iade); free(l->ilade);
    }
    for (int p = 0; p < e->nprobes; ++p) {
        free(e->probes[p].series); free(e->probes[p].freqs); free(e->probes[p].dft);
    }
    for (int d = 0; d < e->ndumps; ++d) {
        dump_t *q = &e->dumps[d];
        free(q->freqs); free(q->acc); free(q->samp_ts); free(q->samples); free(q->rho);
        for (int n = 0; n < 3; ++n) { free(q->el[n]); free(q->del[n]); }
    }
    free(e);
}

const char *oems_ref_last_error(const eng_t *e)
{
    return e ? e->err : "null engine";
}

/* ------------------------------------------------------------------------------------------ */
/* operator */

/* 4-lane compression key: 12 f4 vectors (vv,vi,iv,ii x 3), bitwise equality like SSE_coeff::operator== */
typedef struct {
    uint32_t w[48];
} ckey_t;

static uint64_t key_hash(const ckey_t *k)
{
    uint64_t h = 1469598103934665603ULL;
    for (int i = 0; i < 48; ++i) {
        h ^= k->w[i];
        h *= 1099511628211ULL;
        h ^= h >> 29;
    }
    return h;
}

static int compress_mt(eng_t *e, const float *vv, const float *vi, const float *ii, const float *iv)
{
    unsigned Nx = e->N[0], Ny = e->N[1], Nz = e->N[2], nv = e->nv;
    size_t nvecpos = (size_t)Nx * Ny * nv;
    e->op_index = (unsigned *)xcalloc(nvecpos, sizeof(unsigned));
    size_t cap = 1024, used = 0;
    ckey_t *keys = (ckey_t *)malloc(cap * sizeof(ckey_t));
    size_t hcap = 1 << 16;
    int64_t *htab = (int64_t *)malloc(hcap * sizeof(int64_t));
    if (!e->op_index || !keys || !htab)
        return ERR_NOMEM;
    for (size_t i = 0; i < hcap; ++i)
        htab[i] = -1;
    const float *arr[4] = {vv, vi, iv, ii};
    ckey_t k;
    for (unsigned x = 0; x < Nx; ++x)
        for (unsigned y = 0; y < Ny; ++y)
            for (unsigned v = 0; v < nv; ++v) {
                for (int a = 0; a < 4; ++a)
                    for (int n = 0; n < 3; ++n)
                        for (int l = 0; l < 4; ++l) {
                            unsigned z = v + l * nv;
                            float val = 0.0f; /* lanes beyond Nz stay zero (Operator_sse::InitOperator) */
                            if (z < Nz)
                                val = arr[a][nijk(e, n, x, y, z)];
                            memcpy(&k.w[(a * 3 + n) * 4 + l], &val, 4);
                        }
                uint64_t h = key_hash(&k);
                size_t slot = h & (hcap - 1);
                int64_t found = -1;
                while (htab[slot] >= 0) {
                    if (memcmp(&keys[htab[slot]], &k, sizeof(ckey_t)) == 0) {
                        found = htab[slot];
                        break;
                    }
                    slot = (slot + 1) & (hcap - 1);
                }
                if (found < 0) {
                    if (used == cap) {
                        cap *= 2;
                        keys = (ckey_t *)realloc(keys, cap * sizeof(ckey_t));
                        if (!keys)
                            return ERR_NOMEM;
                    }
                    keys[used] = k;
                    htab[slot] = (int64_t)used;
                    found = (int64_t)used++;
                    if (used * 2 > hcap) { /* rehash */
                        free(htab);
                        hcap *= 4;
                        htab = (int64_t *)malloc(hcap * sizeof(int64_t));
                        if (!htab)
                            return ERR_NOMEM;
                        for (size_t i = 0; i < hcap; ++i)
                            htab[i] = -1;
                        for (size_t j = 0; j < used; ++j) {
                            size_t s2 = key_hash(&keys[j]) & (hcap - 1);
                            while (htab[s2] >= 0)
                                s2 = (s2 + 1) & (hcap - 1);
                            htab[s2] = (int64_t)j;
                        }
                    }
                }
                e->op_index[((size_t)x * Ny + y) * nv + v] = (unsigned)found;
            }
    e->nclasses = (unsigned)used;
    e->cvv = (v4sf *)aligned_alloc(16, 3 * used * sizeof(v4sf) + 16);
    e->cvi = (v4sf *)aligned_alloc(16, 3 * used * sizeof(v4sf) + 16);
    e->cii = (v4sf *)aligned_alloc(16, 3 * used * sizeof(v4sf) + 16);
    e->civ = (v4sf *)aligned_alloc(16, 3 * used * sizeof(v4sf) + 16);
    if (!e->cvv || !e->cvi || !e->cii || !e->civ)
        return ERR_NOMEM;
    v4sf *tabs[4] = {e->cvv, e->cvi, e->civ, e->cii};
    for (size_t j = 0; j < used; ++j)
        for (int a = 0; a < 4; ++a)
            for (int n = 0; n < 3; ++n)
                memcpy(&tabs[a][n * used + j], &keys[j].w[(a * 3 + n) * 4], 16);
    free(keys);
    free(htab);
    return OK;
}

int oems_ref_set_operator(eng_t *e, const float *vv, const float *vi, const float *ii, const float *iv,
                          unsigned max_classes)
{
    (void)max_classes;
    if (!e || !vv || !vi || !ii || !iv)
        return ERR_ARG;
    if (e->mt)
        return compress_mt(e, vv, vi, ii, iv);
    size_t n = 3 * e->cells;
    free(e->vv); free(e->vi); free(e->ii); free(e->iv);
    e->vv = dupf(vv, n); e->vi = dupf(vi, n); e->ii = dupf(ii, n); e->iv = dupf(iv, n);
    return (e->vv && e->vi && e->ii && e->iv) ? OK : ERR_NOMEM;
}

int oems_ref_operator_classes(const eng_t *e, unsigned *nc)
{
    if (!e || !nc)
        return ERR_ARG;
    *nc = e->mt ? e->nclasses : 0;
    return OK;
}

/* ------------------------------------------------------------------------------------------ */
/* extensions: setup */

int oems_ref_set_excitation(eng_t *e, unsigned nV, const unsigned *v_idx, const unsigned short *v_dir,
                            const float *v_amp, const unsigned *v_delay, unsigned nI, const unsigned *i_idx,
                            const unsigned short *i_dir, const float *i_amp, const unsigned *i_delay,
                            const float *sig_v, const float *sig_i, unsigned length, unsigned period)
{
    if (!e || (length && (!sig_v || !sig_i)))
        return ERR_ARG;
    for (unsigned k = 0; k < nV; ++k)
        for (int a = 0; a < 3; ++a)
            if (v_idx[a * nV + k] >= e->N[a] || v_dir[k] > 2)
                return ERR_ARG;
    for (unsigned k = 0; k < nI; ++k)
        for (int a = 0; a < 3; ++a)
            if (i_idx[a * nI + k] >= e->N[a] || i_dir[k] > 2)
                return ERR_ARG;
    e->nV = nV; e->nI = nI; e->sig_len = length; e->period = period;
    e->v_idx = (unsigned *)xcalloc(3 * (size_t)nV, 4); memcpy(e->v_idx, v_idx, 12 * (size_t)nV);
    e->i_idx = (unsigned *)xcalloc(3 * (size_t)nI, 4); if (nI) memcpy(e->i_idx, i_idx, 12 * (size_t)nI);
    e->v_dir = (unsigned short *)xcalloc(nV, 2); if (nV) memcpy(e->v_dir, v_dir, 2 * (size_t)nV);
    e->i_dir = (unsigned short *)xcalloc(nI, 2); if (nI) memcpy(e->i_dir, i_dir, 2 * (size_t)nI);
    e->v_amp = dupf(v_amp, nV); e->i_amp = dupf(i_amp, nI);
    e->v_delay = (unsigned *)xcalloc(nV, 4); if (nV) memcpy(e->v_delay, v_delay, 4 * (size_t)nV);
    e->i_delay = (unsigned *)xcalloc(nI, 4); if (nI) memcpy(e->i_delay, i_delay, 4 * (size_t)nI);
    e->sig_v = dupf(sig_v, length); e->sig_i = dupf(sig_i, length);
    return OK;
}

static void *dupmem(const void *src, size_t bytes)
{
    void *p = xcalloc(bytes ? bytes : 1, 1);
    if (bytes)
        memcpy(p, src, bytes);
    return p;
}

/* Operator_Ext_Cylinder's tables (FDTD/extensions/operator_ext_cylinder.cpp:44-112): a closed
 * alpha mesh and, with rho = 0 on it, vv_r0/vi_r0 for every z line */
int oems_ref_set_cylinder(eng_t *e, int closed_alpha, int r0_included, const float *vv_r0, const float *vi_r0)
{
    if (!e || (r0_included && (!closed_alpha || !vv_r0 || !vi_r0)) || e->N[1] < 3)
        return ERR_ARG;
    e->cyl_closed = closed_alpha != 0;
    e->cyl_r0 = r0_included != 0;
    free(e->cyl_vv_r0); free(e->cyl_vi_r0);
    e->cyl_vv_r0 = e->cyl_vi_r0 = NULL;
    if (e->cyl_r0) {
        e->cyl_vv_r0 = (float *)dupmem(vv_r0, 4 * (size_t)e->N[2]);
        e->cyl_vi_r0 = (float *)dupmem(vi_r0, 4 * (size_t)e->N[2]);
    }
    return OK;
}

int oems_ref_set_tfsf(eng_t *e, unsigned nV, const unsigned *v_idx, const unsigned short *v_dir,
                      const unsigned *v_delay, const float *v_delta, const float *v_amp, unsigned nI,
                      const unsigned *i_idx, const unsigned short *i_dir, const unsigned *i_delay,
                      const float *i_delta, const float *i_amp, const float *sig_v, const float *sig_i,
                      unsigned length, unsigned period, unsigned max_delay)
{
    if (!e || !length || !sig_v || !sig_i || period > length)
        return ERR_ARG;
    if (e->inited)
        return ERR_STATE;
    for (int w = 0; w < 2; ++w) {
        unsigned n = w ? nI : nV;
        const unsigned *idx = w ? i_idx : v_idx, *dl = w ? i_delay : v_delay;
        const unsigned short *dr = w ? i_dir : v_dir;
        for (unsigned k = 0; k < n; ++k)
            if (idx[k] >= e->N[0] || idx[n + k] >= e->N[1] || idx[2 * n + k] >= e->N[2] || dr[k] > 2 ||
                dl[k] >= max_delay)
                return ERR_ARG;
    }
    e->tf_nV = nV;
    e->tf_nI = nI;
    e->tf_v_idx = (unsigned *)dupmem(v_idx, 12 * (size_t)nV);
    e->tf_i_idx = (unsigned *)dupmem(i_idx, 12 * (size_t)nI);
    e->tf_v_dir = (unsigned short *)dupmem(v_dir, 2 * (size_t)nV);
    e->tf_i_dir = (unsigned short *)dupmem(i_dir, 2 * (size_t)nI);
    e->tf_v_delay = (unsigned *)dupmem(v_delay, 4 * (size_t)nV);
    e->tf_i_delay = (unsigned *)dupmem(i_delay, 4 * (size_t)nI);
    e->tf_v_delta = (float *)dupmem(v_delta, 4 * (size_t)nV);
    e->tf_i_delta = (float *)dupmem(i_delta, 4 * (size_t)nI);
    e->tf_v_amp = (float *)dupmem(v_amp, 4 * (size_t)nV);
    e->tf_i_amp = (float *)dupmem(i_amp, 4 * (size_t)nI);
    e->tf_sig_v = (float *)dupmem(sig_v, 4 * (size_t)length);
    e->tf_sig_i = (float *)dupmem(sig_i, 4 * (size_t)length);
    e->tf_lut = (unsigned *)xcalloc((size_t)max_delay + 1, 4);
    e->tf_len = length;
    e->tf_period = period;
    e->tf_max_delay = max_delay;
    return OK;
}

int oems_ref_set_lumped_rlc(eng_t *e, unsigned n, const unsigned *pos, const int *dir, const float *ilv,
                            const float *i2v, const float *vv2, const float *vj1, const float *vj2,
                            const float *vvd, const float *ib0, const float *b1, const float *b2)
{
    if (!e)
        return ERR_ARG;
    if (e->inited)
        return ERR_STATE;
    for (unsigned k = 0; k < n; ++k)
        if (pos[k] >= e->N[0] || pos[n + k] >= e->N[1] || pos[2 * n + k] >= e->N[2] || dir[k] < 0 || dir[k] > 2)
            return ERR_ARG;
    e->rlc_n = n;
    e->rlc_pos = (unsigned *)dupmem(pos, 12 * (size_t)n);
    e->rlc_dir = (int *)dupmem(dir, 4 * (size_t)n);
    e->rlc_c = (float *)xcalloc(9 * (size_t)n + 1, 4);
    const float *src[9] = {ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2};
    for (int q = 0; q < 9; ++q)
        memcpy(e->rlc_c + (size_t)q * n, src[q], 4 * (size_t)n);
    e->rlc_il = (float *)xcalloc((size_t)n + 1, 4);
    for (int q = 0; q < 3; ++q) {
        e->rlc_vd[q] = (float *)xcalloc((size_t)n + 1, 4);
        e->rlc_j[q] = (float *)xcalloc((size_t)n + 1, 4);
    }
    return OK;
}

int oems_ref_add_upml(eng_t *e, const unsigned start[3], const unsigned nl[3], const float *vv,
                      const float *vvfo, const float *vvfn, const float *ii, const float *iifo, const float *iifn)
{
    if (!e || e->nupml >= MAX_UPML)
        return ERR_ARG;
    for (int a = 0; a < 3; ++a)
        if (start[a] + nl[a] > e->N[a] || nl[a] == 0)
            return ERR_ARG;
    upml_t *u = &e->upml[e->nupml++];
    memcpy(u->start, start, 12);
    memcpy(u->nl, nl, 12);
    u->n = (size_t)nl[0] * nl[1] * nl[2];
    size_t m = 3 * u->n;
    u->vv = dupf(vv, m); u->vvfo = dupf(vvfo, m); u->vvfn = dupf(vvfn, m);
    u->ii = dupf(ii, m); u->iifo = dupf(iifo, m); u->iifn = dupf(iifn, m);
    u->vflux = (float *)xcalloc(m, 4);
    u->iflux = (float *)xcalloc(m, 4);
    return OK;
}

int oems_ref_add_mur(eng_t *e, int ny, unsigned line, unsigned shift, unsigned start_ts, const float *cP,
                     const float *cPP)
{
    if (!e || e->nmur >= MAX_MUR || ny < 0 || ny > 2 || line >= e->N[ny] || shift >= e->N[ny])
        return ERR_ARG;
    mur_t *m = &e->mur[e->nmur++];
    m->ny = ny; m->nyP = (ny + 1) % 3; m->nyPP = (ny + 2) % 3;
    m->line = line; m->shift = shift; m->start_ts = start_ts;
    m->n1 = e->N[m->nyP]; m->n2 = e->N[m->nyPP];
    size_t n = (size_t)m->n1 * m->n2;
    m->cP = dupf(cP, n); m->cPP = dupf(cPP, n);
    m->bP = (float *)xcalloc(n, 4); m->bPP = (float *)xcalloc(n, 4);
    return OK;
}

int oems_ref_add_lorentz_order(eng_t *e, unsigned count, const unsigned *pos, int von, int con, int vlon,
                               int clon, const float *vint, const float *vext, const float *vlor,
                               const float *iint, const float *iext, const float *ilor)
{
    if (!e || e->nlor >= MAX_LOR)
        return ERR_ARG;
    for (unsigned i = 0; i < count; ++i)
        for (int a = 0; a < 3; ++a)
            if (pos[a * count + i] >= e->N[a])
                return ERR_ARG;
    lor_t *l = &e->lor[e->nlor++];
    size_t m = 3 * (size_t)count;
    l->count = count;
    l->pos = (unsigned *)xcalloc(m, 4);
    if (count) memcpy(l->pos, pos, 4 * m);
    l->von = von; l->con = con; l->vlon = vlon && von; l->clon = clon && con;
    l->vint = von ? dupf(vint, m) : NULL; l->vext = von ? dupf(vext, m) : NULL;
    l->vlor = l->vlon ? dupf(vlor, m) : NULL;
    l->iint = con ? dupf(iint, m) : NULL; l->iext = con ? dupf(iext, m) : NULL;
    l->ilor = l->clon ? dupf(ilor, m) : NULL;
    l->vade = von ? (float *)xcalloc(m, 4) : NULL;
    l->vlade = l->vlon ? (float *)xcalloc(m, 4) : NULL;
    l->iade = con ? (float *)xcalloc(m, 4) : NULL;
    l->ilade = l->clon ? (float *)xcalloc(m, 4) : NULL;
    return OK;
}

static int add_probe(eng_t *e, int type, const unsigned start[3], const unsigned stop[3], int nd, const int si[3],
                     const int ei[3], double weight, unsigned interval, unsigned start_ts, unsigned stop_ts, int *id)
{
    if (!e || e->nprobes >= MAX_PROBES || !id)
        return ERR_ARG;
    for (int a = 0; a < 3; ++a)
        if (start[a] >= e->N[a] || stop[a] >= e->N[a])
            return ERR_ARG;
    if (type == 0) {
        int diff = (start[0] != stop[0]) + (start[1] != stop[1]) + (start[2] != stop[2]);
        if (diff != 1)
            return ERR_ARG;
    } else if (type == 1 && (nd < 0 || nd > 2))
        return ERR_ARG;
    probe_t *p = &e->probes[e->nprobes];
    memset(p, 0, sizeof(*p));
    p->type = type;
    p->ncomp = type >= 2 ? 3 : 1;
    memcpy(p->start, start, 12);
    memcpy(p->stop, stop, 12);
    p->nd = nd;
    for (int a = 0; a < 3; ++a) {
        p->si[a] = si ? si[a] : 1;
        p->ei[a] = ei ? ei[a] : 1;
    }
    p->weight = weight;
    p->interval = interval ? interval : 1;
    p->start_ts = start_ts;
    p->stop_ts = stop_ts;
    *id = e->nprobes++;
    return OK;
}

int oems_ref_add_voltage_probe(eng_t *e, const unsigned start[3], const unsigned stop[3], double weight,
                               unsigned interval, unsigned start_ts, unsigned stop_ts, int *id)
{
    return add_probe(e, 0, start, stop, -1, NULL, NULL, weight, interval, start_ts, stop_ts, id);
}

int oems_ref_add_current_probe(eng_t *e, const unsigned start[3], const unsigned stop[3], int nd, const int si[3],
                               const int ei[3], double weight, unsigned interval, unsigned start_ts, unsigned stop_ts,
                               int *id)
{
    return add_probe(e, 1, start, stop, nd, si, ei, weight, interval, start_ts, stop_ts, id);
}

/* ProcessFieldProbe (Common/processfieldprobe.cpp:77-92): the E (field 0) or H (field 1) field
 * at one Yee position without interpolation; el = the three edge lengths there */
int oems_ref_add_field_probe(eng_t *e, int field, const unsigned pos[3], const double el[3], double weight,
                             unsigned interval, unsigned start_ts, unsigned stop_ts, int *id)
{
    if (!e || !el || (field != 0 && field != 1))
        return ERR_ARG;
    int rc = add_probe(e, 2 + field, pos, pos, -1, NULL, NULL, weight, interval, start_ts, stop_ts, id);
    if (rc == OK)
        memcpy(e->probes[*id].el, el, sizeof(double) * 3);
    return rc;
}

int oems_ref_set_probe_dft(eng_t *e, int id, unsigned fd_interval, unsigned nf, const double *freqs)
{
    if (!e || id < 0 || id >= e->nprobes || (nf && !freqs))
        return ERR_ARG;
    probe_t *p = &e->probes[id];
    p->fd_interval = fd_interval;
    p->nf = nf;
    free(p->freqs); free(p->dft);
    p->freqs = (double *)xcalloc(nf, 8);
    if (nf) memcpy(p->freqs, freqs, 8 * (size_t)nf);
    p->dft = (double *)xcalloc(2 * (size_t)nf * p->ncomp, 8);
    return OK;
}

/* A dump on a cylindrical mesh (no interpolation only): rho of every x line of the dump's mesh
 * (main for E, dual for H), which scales the alpha edge lengths */
int oems_ref_set_dump_rho(eng_t *e, int id, const double *rho)
{
    if (!e || id < 0 || id >= e->ndumps || !rho || e->dumps[id].interp != 0)
        return ERR_ARG;
    free(e->dumps[id].rho);
    e->dumps[id].rho = (double *)dupmem(rho, 8 * (size_t)e->N[0]);
    return OK;
}

int oems_ref_add_fd_dump(eng_t *e, int field, int interp, const unsigned start[3], const unsigned stop[3],
                         unsigned fd_interval, unsigned nf, const double *freqs, const double *el, const double *del,
                         int *id)
{
    if (!e || e->ndumps >= MAX_DUMPS || (field != 0 && field != 1) || !id || !el || !del || interp < 0 || interp > 2)
        return ERR_ARG;
    dump_t *d = &e->dumps[e->ndumps];
    memset(d, 0, sizeof(*d));
    d->field = field;
    d->interp = interp;
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        if (start[a] > stop[a] || stop[a] >= e->N[a])
            return ERR_ARG;
        d->start[a] = start[a];
        d->stop[a] = stop[a];
        d->sz[a] = stop[a] - start[a] + 1;
        d->el[a] = (double *)xcalloc(e->N[a], 8);
        d->del[a] = (double *)xcalloc(e->N[a], 8);
        memcpy(d->el[a], el + off, 8 * (size_t)e->N[a]);
        memcpy(d->del[a], del + off, 8 * (size_t)e->N[a]);
        off += e->N[a];
    }
    d->fd_interval = fd_interval;
    d->nf = nf;
    d->freqs = (double *)xcalloc(nf, 8);
    if (nf) memcpy(d->freqs, freqs, 8 * (size_t)nf);
    d->acc = (float *)xcalloc((size_t)nf * 3 * d->sz[0] * d->sz[1] * d->sz[2] * 2, 4);
    *id = e->ndumps++;
    return OK;
}

/* same arguments as oems_cuda_add_td_dump; the oracle keeps the samples in memory (coords and
 * file_prefix are unused) and serves them through oems_ref_read_td_sample */
int oems_ref_add_td_dump(eng_t *e, int field, int interp, const unsigned start[3], const unsigned stop[3],
                         unsigned interval, unsigned start_ts, unsigned stop_ts, const double *el, const double *del,
                         const double *coords, const char *file_prefix, int *id)
{
    (void)coords;
    (void)file_prefix;
    if (!interval)
        return ERR_ARG;
    int rc = oems_ref_add_fd_dump(e, field, interp, start, stop, 0, 0, NULL, el, del, id);
    if (rc)
        return rc;
    dump_t *d = &e->dumps[*id];
    d->td = 1;
    d->td_interval = interval;
    d->td_start = start_ts;
    d->td_stop = stop_ts;
    return OK;
}

/* number of samples through *count; sample k (if out != NULL) as float [3][sx][sy][sz] with its step */
int oems_ref_read_td_sample(const eng_t *e, int id, unsigned k, float *out, unsigned *ts, unsigned *count)
{
    if (!e || id < 0 || id >= e->ndumps || !e->dumps[id].td)
        return ERR_ARG;
    const dump_t *d = &e->dumps[id];
    if (count)
        *count = d->nsamp;
    if (!out)
        return OK;
    if (k >= d->nsamp)
        return ERR_ARG;
    size_t plane = (size_t)d->sz[0] * d->sz[1] * d->sz[2];
    memcpy(out, d->samples + (size_t)k * 3 * plane, 12 * plane);
    if (ts)
        *ts = d->samp_ts[k];
    return OK;
}

/* ------------------------------------------------------------------------------------------ */
/* basic engine update: Engine::UpdateVoltages / UpdateCurrents (FDTD/engine.cpp:110-222) */

static void update_voltages_basic(eng_t *e, unsigned startX, unsigned numX)
{
    const unsigned Ny = e->N[1], Nz = e->N[2];
    float *V = e->volt;
    const float *I = e->curr;
    const float *vv = e->vv, *vi = e->vi;
    unsigned pos0 = startX;
    for (unsigned px = 0; px < numX; ++px, ++pos0) {
        unsigned s0 = pos0 ? 1 : 0;
        for (unsigned y = 0; y < Ny; ++y) {
            unsigned s1 = y ? 1 : 0;
            for (unsigned z = 0; z < Nz; ++z) {
                unsigned s2 = z ? 1 : 0;
                size_t i0 = nijk(e, 0, pos0, y, z), i1 = nijk(e, 1, pos0, y, z), i2 = nijk(e, 2, pos0, y, z);
                float t;
                /* x */
                V[i0] *= vv[i0];
                t = I[i2] - I[nijk(e, 2, pos0, y - s1, z)];
                t = t - I[i1];
                t = t + I[nijk(e, 1, pos0, y, z - s2)];
                V[i0] += vi[i0] * t;
                /* y */
                V[i1] *= vv[i1];
                t = I[i0] - I[nijk(e, 0, pos0, y, z - s2)];
                t = t - I[i2];
                t = t + I[nijk(e, 2, pos0 - s0, y, z)];
                V[i1] += vi[i1] * t;
                /* z */
                V[i2] *= vv[i2];
                t = I[i1] - I[nijk(e, 1, pos0 - s0, y, z)];
                t = t - I[i0];
                t = t + I[nijk(e, 0, pos0, y - s1, z)];
                V[i2] += vi[i2] * t;
            }
        }
    }
}

static void update_currents_basic(eng_t *e, unsigned startX, unsigned numX)
{
    const unsigned Ny = e->N[1], Nz = e->N[2];
    float *I = e->curr;
    const float *V = e->volt;
    const float *ii = e->ii, *iv = e->iv;
    unsigned pos0 = startX;
    for (unsigned px = 0; px < numX; ++px, ++pos0) {
        for (unsigned y = 0; y + 1 < Ny; ++y) {
            for (unsigned z = 0; z + 1 < Nz; ++z) {
                size_t i0 = nijk(e, 0, pos0, y, z), i1 = nijk(e, 1, pos0, y, z), i2 = nijk(e, 2, pos0, y, z);
                float t;
                I[i0] *= ii[i0];
                t = V[i2] - V[nijk(e, 2, pos0, y + 1, z)];
                t = t - V[i1];
                t = t + V[nijk(e, 1, pos0, y, z + 1)];
                I[i0] += iv[i0] * t;
                I[i1] *= ii[i1];
                t = V[i0] - V[nijk(e, 0, pos0, y, z + 1)];
                t = t - V[i2];
                t = t + V[nijk(e, 2, pos0 + 1, y, z)];
                I[i1] += iv[i1] * t;
                I[i2] *= ii[i2];
                t = V[i1] - V[nijk(e, 1, pos0 + 1, y, z)];
                t = t - V[i0];
                t = t + V[nijk(e, 0, pos0, y + 1, z)];
                I[i2] += iv[i2] * t;
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* SSE-compressed update (FDTD/engine_sse_compressed.cpp:51-311), lane-strided 4-lane vectors. */

static inline v4sf lane_up(v4sf a) /* _mm_slli_si128(a,4): lane0 = 0, lane k = a[k-1] */
{
    v4sf r = {0.0f, a[0], a[1], a[2]};
    return r;
}

static inline v4sf lane_down(v4sf a) /* _mm_srli_si128(a,4): lane k = a[k+1], lane3 = 0 */
{
    v4sf r = {a[1], a[2], a[3], 0.0f};
    return r;
}

static void update_voltages_mt(eng_t *e, unsigned startX, unsigned numX)
{
    const unsigned Ny = e->N[1], nv = e->nv, U = e->nclasses;
    v4sf *V = e->f4volt;
    const v4sf *I = e->f4curr;
    const size_t sx = (size_t)Ny * nv * 3, sy = (size_t)nv * 3, sz = 3;
    unsigned pos0 = startX;
    for (unsigned px = 0; px < numX; ++px, ++pos0) {
        size_t ix = pos0 > 0 ? sx : 0;
        for (unsigned y = 0; y < Ny; ++y) {
            size_t iy = y > 0 ? sy : 0;
            size_t row = ((size_t)pos0 * Ny + y) * nv;
            for (unsigned v = 1; v < nv; ++v) {
                unsigned c = e->op_index[row + v];
                size_t p = (row + v) * 3;
                V[p + 0] = V[p + 0] * e->cvv[0 * U + c];
                V[p + 0] = V[p + 0] + e->cvi[0 * U + c] * (((I[p + 2] - I[p + 2 - iy]) - I[p + 1]) + I[p + 1 - sz]);
                V[p + 1] = V[p + 1] * e->cvv[1 * U + c];
                V[p + 1] = V[p + 1] + e->cvi[1 * U + c] * (((I[p + 0] - I[p + 0 - sz]) - I[p + 2]) + I[p + 2 - ix]);
                V[p + 2] = V[p + 2] * e->cvv[2 * U + c];
                V[p + 2] = V[p + 2] + e->cvi[2 * U + c] * (((I[p + 1] - I[p + 1 - ix]) - I[p + 0]) + I[p + 0 - iy]);
            }
            /* vector 0: the z-1 neighbour is vector nv-1 shifted up one lane */
            {
                unsigned c = e->op_index[row];
                size_t p = row * 3, pe = (row + nv - 1) * 3;
                v4sf t = lane_up(I[pe + 1]);
                V[p + 0] = V[p + 0] * e->cvv[0 * U + c];
                V[p + 0] = V[p + 0] + e->cvi[0 * U + c] * (((I[p + 2] - I[p + 2 - iy]) - I[p + 1]) + t);
                t = lane_up(I[pe + 0]);
                V[p + 1] = V[p + 1] * e->cvv[1 * U + c];
                V[p + 1] = V[p + 1] + e->cvi[1 * U + c] * (((I[p + 0] - t) - I[p + 2]) + I[p + 2 - ix]);
                V[p + 2] = V[p + 2] * e->cvv[2 * U + c];
                V[p + 2] = V[p + 2] + e->cvi[2 * U + c] * (((I[p + 1] - I[p + 1 - ix]) - I[p + 0]) + I[p + 0 - iy]);
            }
        }
    }
}

static void update_currents_mt(eng_t *e, unsigned startX, unsigned numX)
{
    const unsigned Ny = e->N[1], nv = e->nv, U = e->nclasses;
    const v4sf *V = e->f4volt;
    v4sf *I = e->f4curr;
    const size_t sx = (size_t)Ny * nv * 3, sy = (size_t)nv * 3, sz = 3;
    unsigned pos0 = startX;
    for (unsigned px = 0; px < numX; ++px, ++pos0) {
        for (unsigned y = 0; y + 1 < Ny; ++y) {
            size_t row = ((size_t)pos0 * Ny + y) * nv;
            for (unsigned v = 0; v + 1 < nv; ++v) {
                unsigned c = e->op_index[row + v];
                size_t p = (row + v) * 3;
                I[p + 0] = I[p + 0] * e->cii[0 * U + c];
                I[p + 0] = I[p + 0] + e->civ[0 * U + c] * (((V[p + 2] - V[p + 2 + sy]) - V[p + 1]) + V[p + 1 + sz]);
                I[p + 1] = I[p + 1] * e->cii[1 * U + c];
                I[p + 1] = I[p + 1] + e->civ[1 * U + c] * (((V[p + 0] - V[p + 0 + sz]) - V[p + 2]) + V[p + 2 + sx]);
                I[p + 2] = I[p + 2] * e->cii[2 * U + c];
                I[p + 2] = I[p + 2] + e->civ[2 * U + c] * (((V[p + 1] - V[p + 1 + sx]) - V[p + 0]) + V[p + 0 + sy]);
            }
            /* last vector: the z+1 neighbour is vector 0 shifted down one lane */
            {
                unsigned c = e->op_index[row + nv - 1];
                size_t p = (row + nv - 1) * 3, ps = row * 3;
                v4sf t = lane_down(V[ps + 1]);
                I[p + 0] = I[p + 0] * e->cii[0 * U + c];
                I[p + 0] = I[p + 0] + e->civ[0 * U + c] * (((V[p + 2] - V[p + 2 + sy]) - V[p + 1]) + t);
                t = lane_down(V[ps + 0]);
                I[p + 1] = I[p + 1] * e->cii[1 * U + c];
                I[p + 1] = I[p + 1] + e->civ[1 * U + c] * (((V[p + 0] - t) - V[p + 2]) + V[p + 2 + sx]);
                I[p + 2] = I[p + 2] * e->cii[2 * U + c];
                I[p + 2] = I[p + 2] + e->civ[2 * U + c] * (((V[p + 1] - V[p + 1 + sx]) - V[p + 0]) + V[p + 0 + sy]);
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* extension hooks (accessor based, like the reference's templated Impl functions) */

/* Engine_Ext_LorentzMaterial::DoPreVoltageUpdatesImpl (engine_ext_lorentzmaterial.cpp:79-120) */
static void lorentz_pre_volt(eng_t *e, lor_t *l)
{
    if (!l->von)
        return;
    unsigned M = l->count;
    for (unsigned i = 0; i < M; ++i) {
        unsigned x = l->pos[i], y = l->pos[M + i], z = l->pos[2 * M + i];
        for (int n = 0; n < 3; ++n) {
            size_t k = (size_t)n * M + i;
            float vol = GETV(e, n, x, y, z);
            if (l->vlon) {
                l->vlade[k] += l->vlor[k] * l->vade[k];
                l->vade[k] *= l->vint[k];
                l->vade[k] += l->vext[k] * (vol - l->vlade[k]);
            } else {
                l->vade[k] *= l->vint[k];
                l->vade[k] += l->vext[k] * vol;
            }
        }
    }
}

static void lorentz_pre_curr(eng_t *e, lor_t *l)
{
    if (!l->con)
        return;
    unsigned M = l->count;
    for (unsigned i = 0; i < M; ++i) {
        unsigned x = l->pos[i], y = l->pos[M + i], z = l->pos[2 * M + i];
        for (int n = 0; n < 3; ++n) {
            size_t k = (size_t)n * M + i;
            float cur = GETI(e, n, x, y, z);
            if (l->clon) {
                l->ilade[k] += l->ilor[k] * l->iade[k];
                l->iade[k] *= l->iint[k];
                l->iade[k] += l->iext[k] * (cur - l->ilade[k]);
            } else {
                l->iade[k] *= l->iint[k];
                l->iade[k] += l->iext[k] * cur;
            }
        }
    }
}

/* Engine_Ext_Dispersive::Apply2VoltagesImpl / Apply2CurrentImpl (engine_ext_dispersive.cpp:76-127) */
static void lorentz_apply(eng_t *e, lor_t *l, int curr)
{
    if (curr ? !l->con : !l->von)
        return;
    unsigned M = l->count;
    float *ade = curr ? l->iade : l->vade;
    for (unsigned i = 0; i < M; ++i) {
        unsigned x = l->pos[i], y = l->pos[M + i], z = l->pos[2 * M + i];
        for (int n = 0; n < 3; ++n) {
            float *f = fptr(e, curr, n, x, y, z);
            *f = *f - ade[(size_t)n * M + i];
        }
    }
}

/* Engine_Ext_Mur_ABC (engine_ext_mur_abc.cpp:82-178) */
static int mur_active(const eng_t *e, const mur_t *m)
{
    return e->numTS >= m->start_ts;
}

static void mur_pre(eng_t *e, mur_t *m)
{
    if (!mur_active(e, m))
        return;
    unsigned pos[3] = {0, 0, 0}, ps[3] = {0, 0, 0};
    pos[m->ny] = m->line;
    ps[m->ny] = m->shift;
    for (unsigned i = 0; i < m->n1; ++i) {
        pos[m->nyP] = ps[m->nyP] = i;
        for (unsigned j = 0; j < m->n2; ++j) {
            pos[m->nyPP] = ps[m->nyPP] = j;
            size_t k = (size_t)i * m->n2 + j;
            m->bP[k] = GETV(e, m->nyP, ps[0], ps[1], ps[2]) - m->cP[k] * GETV(e, m->nyP, pos[0], pos[1], pos[2]);
            m->bPP[k] = GETV(e, m->nyPP, ps[0], ps[1], ps[2]) - m->cPP[k] * GETV(e, m->nyPP, pos[0], pos[1], pos[2]);
        }
    }
}

static void mur_post(eng_t *e, mur_t *m)
{
    if (!mur_active(e, m))
        return;
    unsigned ps[3] = {0, 0, 0};
    ps[m->ny] = m->shift;
    for (unsigned i = 0; i < m->n1; ++i) {
        ps[m->nyP] = i;
        for (unsigned j = 0; j < m->n2; ++j) {
            ps[m->nyPP] = j;
            size_t k = (size_t)i * m->n2 + j;
            m->bP[k] += m->cP[k] * GETV(e, m->nyP, ps[0], ps[1], ps[2]);
            m->bPP[k] += m->cPP[k] * GETV(e, m->nyPP, ps[0], ps[1], ps[2]);
        }
    }
}

static void mur_apply(eng_t *e, mur_t *m)
{
    if (!mur_active(e, m))
        return;
    unsigned pos[3] = {0, 0, 0};
    pos[m->ny] = m->line;
    for (unsigned i = 0; i < m->n1; ++i) {
        pos[m->nyP] = i;
        for (unsigned j = 0; j < m->n2; ++j) {
            pos[m->nyPP] = j;
            size_t k = (size_t)i * m->n2 + j;
            GETV(e, m->nyP, pos[0], pos[1], pos[2]) = m->bP[k];
            GETV(e, m->nyPP, pos[0], pos[1], pos[2]) = m->bPP[k];
        }
    }
}

/* Engine_Ext_UPML (engine_ext_upml.cpp:52-229), x-lines [x0, x1) of region u */
static void upml_pre(eng_t *e, upml_t *u, int curr, unsigned x0, unsigned x1)
{
    const float *cv = curr ? u->ii : u->vv, *fo = curr ? u->iifo : u->vvfo;
    float *flux = curr ? u->iflux : u->vflux;
    for (unsigned lx = x0; lx < x1; ++lx)
        for (unsigned ly = 0; ly < u->nl[1]; ++ly)
            for (unsigned lz = 0; lz < u->nl[2]; ++lz)
                for (int n = 0; n < 3; ++n) {
                    size_t k = (((size_t)n * u->nl[0] + lx) * u->nl[1] + ly) * u->nl[2] + lz;
                    float *f = fptr(e, curr, n, lx + u->start[0], ly + u->start[1], lz + u->start[2]);
                    float h = cv[k] * *f - fo[k] * flux[k];
                    *f = flux[k];
                    flux[k] = h;
                }
}

static void upml_post(eng_t *e, upml_t *u, int curr, unsigned x0, unsigned x1)
{
    const float *fn = curr ? u->iifn : u->vvfn;
    float *flux = curr ? u->iflux : u->vflux;
    for (unsigned lx = x0; lx < x1; ++lx)
        for (unsigned ly = 0; ly < u->nl[1]; ++ly)
            for (unsigned lz = 0; lz < u->nl[2]; ++lz)
                for (int n = 0; n < 3; ++n) {
                    size_t k = (((size_t)n * u->nl[0] + lx) * u->nl[1] + ly) * u->nl[2] + lz;
                    float *f = fptr(e, curr, n, lx + u->start[0], ly + u->start[1], lz + u->start[2]);
                    float h = flux[k];
                    flux[k] = *f;
                    *f = h + fn[k] * flux[k];
                }
}

/* Engine_Ext_Excitation::Apply2VoltagesImpl / Apply2CurrentImpl (engine_ext_excitation.cpp:33-94) */
static void excitation_apply(eng_t *e, int curr)
{
    unsigned cnt = curr ? e->nI : e->nV;
    if (!cnt || !e->sig_len)
        return;
    int numTS = (int)e->numTS;
    int p = numTS + 1;
    if (e->period > 0)
        p = (int)e->period;
    const unsigned *idx = curr ? e->i_idx : e->v_idx;
    const unsigned *delay = curr ? e->i_delay : e->v_delay;
    const unsigned short *dir = curr ? e->i_dir : e->v_dir;
    const float *amp = curr ? e->i_amp : e->v_amp;
    const float *sig = curr ? e->sig_i : e->sig_v;
    for (unsigned n = 0; n < cnt; ++n) {
        int exc_pos = numTS - (int)delay[n];
        exc_pos *= (exc_pos > 0);
        exc_pos %= p;
        exc_pos *= (exc_pos < (int)e->sig_len);
        float *f = fptr(e, curr, dir[n], idx[n], idx[cnt + n], idx[2 * cnt + n]);
        *f = *f + amp[n] * sig[exc_pos];
    }
}

/* Engine_Ext_TFSF::DoPostVoltageUpdates / DoPostCurrentUpdates (FDTD/extensions/engine_ext_tfsf.cpp:36-215)
 * on the flattened term list (same order as the reference's face/position/component loops).
 * The delay lookup is rebuilt per hook like m_DelayLookup: entries 0..max_delay in the voltage
 * hook, 0..max_delay-1 in the current hook (entry max_delay keeps the voltage hook's value). */
static void tfsf_apply(eng_t *e, int curr)
{
    unsigned cnt = curr ? e->tf_nI : e->tf_nV;
    if (!e->tf_len || (!e->tf_nV && !e->tf_nI))
        return;
    unsigned numTS = e->numTS, length = e->tf_len;
    int p = (int)e->tf_period;
    unsigned top = curr ? e->tf_max_delay : e->tf_max_delay + 1;
    for (unsigned n = 0; n < top; ++n) {
        if (numTS < n)
            e->tf_lut[n] = 0;
        else if ((numTS - n >= length) && (p == 0))
            e->tf_lut[n] = 0;
        else
            e->tf_lut[n] = numTS - n;
        if (p > 0)
            e->tf_lut[n] = (e->tf_lut[n] % p);
    }
    /* the voltage hook adds the current signal, the current hook the voltage signal */
    const float *signal = curr ? e->tf_sig_v : e->tf_sig_i;
    const unsigned *idx = curr ? e->tf_i_idx : e->tf_v_idx;
    const unsigned *delay = curr ? e->tf_i_delay : e->tf_v_delay;
    const unsigned short *dir = curr ? e->tf_i_dir : e->tf_v_dir;
    const float *dd = curr ? e->tf_i_delta : e->tf_v_delta;
    const float *amp = curr ? e->tf_i_amp : e->tf_v_amp;
    for (unsigned k = 0; k < cnt; ++k) {
        float *f = fptr(e, curr, dir[k], idx[k], idx[cnt + k], idx[2 * cnt + k]);
        *f = *f + (1.0 - dd[k]) * amp[k] * signal[e->tf_lut[delay[k]]]
                + dd[k] * amp[k] * signal[e->tf_lut[1 + delay[k]]];
    }
}

/* Engine_Ext_LumpedRLC::DoPreVoltageUpdates (FDTD/extensions/engine_ext_lumpedRLC.cpp:80-95) */
static void rlc_pre(eng_t *e)
{
    if (!e->rlc_n)
        return;
    float *t = e->rlc_vd[2];
    e->rlc_vd[2] = e->rlc_vd[1];
    e->rlc_vd[1] = e->rlc_vd[0];
    e->rlc_vd[0] = t;
    unsigned n = e->rlc_n;
    const float *ilv = e->rlc_c, *i2v = e->rlc_c + n;
    for (unsigned k = 0; k < n; ++k)
        e->rlc_il[k] += i2v[k] * ilv[k] * e->rlc_vd[1][k];
}

/* Engine_Ext_LumpedRLC::Apply2VoltagesImpl (engine_ext_lumpedRLC.cpp:97-141) */
static void rlc_apply(eng_t *e)
{
    if (!e->rlc_n)
        return;
    float *t = e->rlc_j[2];
    e->rlc_j[2] = e->rlc_j[1];
    e->rlc_j[1] = e->rlc_j[0];
    e->rlc_j[0] = t;
    unsigned n = e->rlc_n;
    const float *c = e->rlc_c;
    const float *vv2 = c + 2 * n, *vj1 = c + 3 * n, *vj2 = c + 4 * n, *vvd = c + 5 * n, *ib0 = c + 6 * n;
    const float *b1 = c + 7 * n, *b2 = c + 8 * n;
    float **Vd = e->rlc_vd, **J = e->rlc_j;
    for (unsigned k = 0; k < n; ++k)
        Vd[0][k] = *fptr(e, 0, e->rlc_dir[k], e->rlc_pos[k], e->rlc_pos[n + k], e->rlc_pos[2 * n + k]);
    for (unsigned k = 0; k < n; ++k) {
        Vd[0][k] = vvd[k] * (Vd[0][k] - e->rlc_il[k] + vv2[k] * Vd[2][k] + vj1[k] * J[1][k] + vj2[k] * J[2][k]);
        J[0][k] = ib0[k] * (Vd[0][k] - Vd[2][k]) - (b1[k] * ib0[k]) * J[1][k] - (b2[k] * ib0[k]) * J[2][k];
    }
    for (unsigned k = 0; k < n; ++k)
        *fptr(e, 0, e->rlc_dir[k], e->rlc_pos[k], e->rlc_pos[n + k], e->rlc_pos[2 * n + k]) = Vd[0][k];
}

/* ------------------------------------------------------------------------------------------ */
/* processing */

/* Engine_Interface_FDTD::CalcVoltageIntegral (FDTD/engine_interface_fdtd.cpp:206-232) */
static double voltage_integral(eng_t *e, const probe_t *p)
{
    double result = 0;
    for (int n = 0; n < 3; ++n) {
        if (p->start[n] < p->stop[n]) {
            unsigned pos[3] = {p->start[0], p->start[1], p->start[2]};
            for (; pos[n] < p->stop[n]; ++pos[n])
                result += GETV(e, n, pos[0], pos[1], pos[2]);
        } else {
            unsigned pos[3] = {p->stop[0], p->stop[1], p->stop[2]};
            for (; pos[n] < p->start[n]; ++pos[n])
                result -= GETV(e, n, pos[0], pos[1], pos[2]);
        }
    }
    return result;
}

/* ProcessCurrent::CalcIntegral (Common/processcurrent.cpp:96-171) */
static double current_integral(eng_t *e, const probe_t *p)
{
    float current = 0;
    const unsigned *s = p->start, *t = p->stop;
    const int *si = p->si, *ei = p->ei;
    unsigned i;
    switch (p->nd) {
    case 0:
        if (ei[0] && si[2]) for (i = s[1] + 1; i <= t[1]; ++i) current += GETI(e, 1, t[0], i, s[2]);
        if (ei[0] && ei[1]) for (i = s[2] + 1; i <= t[2]; ++i) current += GETI(e, 2, t[0], t[1], i);
        if (si[0] && ei[2]) for (i = s[1] + 1; i <= t[1]; ++i) current -= GETI(e, 1, s[0], i, t[2]);
        if (si[0] && si[1]) for (i = s[2] + 1; i <= t[2]; ++i) current -= GETI(e, 2, s[0], s[1], i);
        break;
    case 1:
        if (si[0] && si[1]) for (i = s[2] + 1; i <= t[2]; ++i) current += GETI(e, 2, s[0], s[1], i);
        if (ei[1] && ei[2]) for (i = s[0] + 1; i <= t[0]; ++i) current += GETI(e, 0, i, t[1], t[2]);
        if (ei[0] && ei[1]) for (i = s[2] + 1; i <= t[2]; ++i) current -= GETI(e, 2, t[0], t[1], i);
        if (si[1] && si[2]) for (i = s[0] + 1; i <= t[0]; ++i) current -= GETI(e, 0, i, s[1], s[2]);
        break;
    case 2:
        if (si[1] && si[2]) for (i = s[0] + 1; i <= t[0]; ++i) current += GETI(e, 0, i, s[1], s[2]);
        if (ei[0] && si[2]) for (i = s[1] + 1; i <= t[1]; ++i) current += GETI(e, 1, t[0], i, s[2]);
        if (ei[1] && ei[2]) for (i = s[0] + 1; i <= t[0]; ++i) current -= GETI(e, 0, i, t[1], t[2]);
        if (si[0] && ei[2]) for (i = s[1] + 1; i <= t[1]; ++i) current -= GETI(e, 1, s[0], i, t[2]);
        break;
    default:
        return 0.0;
    }
    return current;
}

/* ProcessIntegral::Process (Common/processintegral.cpp:134-171) */
static void process_probes(eng_t *e)
{
    unsigned ts = e->numTS;
    for (int k = 0; k < e->nprobes; ++k) {
        probe_t *p = &e->probes[k];
        if (ts < p->start_ts || ts > p->stop_ts)
            continue;
        int do_td = (ts % p->interval) == 0;
        int do_fd = p->fd_interval && (ts % p->fd_interval) == 0;
        if (!do_td && !do_fd)
            continue;
        if (p->type >= 2) {
            /* Engine_Interface_FDTD::GetRawField (FDTD/engine_interface_fdtd.cpp:263-276) / GetRawDualField (:136-148):
             * value / edge length, 0 on a zero length; rows of ProcessIntegral::Process per component */
            const unsigned *q = p->start;
            double time = ((double)ts + (double)(p->type == 3) * 0.5) * e->dt;
            for (unsigned c = 0; c < 3; ++c) {
                double value = p->type == 2 ? (double)GETV(e, c, q[0], q[1], q[2]) : (double)GETI(e, c, q[0], q[1], q[2]);
                double v = p->el[c] != 0.0 ? value / p->el[c] : 0.0;
                double a = v * p->weight;
                if (do_td) {
                    size_t slot = ts / p->interval;
                    if (slot < p->nslots)
                        p->series[3 * slot + c] = a;
                }
                if (do_fd) {
                    for (unsigned f = 0; f < p->nf; ++f) {
                        double th = ((-2.0 * M_PI_REF) * p->freqs[f]) * time;
                        double complex ex = cexp(CMPLX(-0.0, th));
                        double re = creal(ex) * a, im = cimag(ex) * a;
                        re = re * 2.0; im = im * 2.0;
                        re = re * e->dt; im = im * e->dt;
                        re = re * (double)p->fd_interval; im = im * (double)p->fd_interval;
                        p->dft[2 * (3 * f + c)] += re;
                        p->dft[2 * (3 * f + c) + 1] += im;
                    }
                }
            }
            continue;
        }
        double val = p->type == 0 ? voltage_integral(e, p) : current_integral(e, p);
        double time = ((double)ts + (double)(p->type == 1) * 0.5) * e->dt;
        if (do_td) {
            size_t slot = ts / p->interval;
            if (slot < p->nslots)
                p->series[slot] = val * p->weight;
        }
        if (do_fd) {
            for (unsigned f = 0; f < p->nf; ++f) {
                double th = ((-2.0 * M_PI_REF) * p->freqs[f]) * time;
                double complex ex = cexp(CMPLX(-0.0, th));
                double a = val * p->weight;
                double re = creal(ex) * a, im = cimag(ex) * a;
                re = re * 2.0; im = im * 2.0;
                re = re * e->dt; im = im * e->dt;
                re = re * (double)p->fd_interval; im = im * (double)p->fd_interval;
                p->dft[2 * f] += re;
                p->dft[2 * f + 1] += im;
            }
        }
    }
}

/* GetRawInterpolatedField / GetRawInterpolatedDualField, CELL_INTERPOLATE
 * (FDTD/engine_interface_fdtd.cpp:104-121, 182-199) */
/* Engine_Interface_FDTD::GetRawInterpolatedField (E, FDTD/engine_interface_fdtd.cpp:63-123) and
 * GetRawInterpolatedDualField (H, :140-204) with the dump's interpolation type */
static void dump_field(eng_t *e, const dump_t *d, const unsigned pos[3], double out[3])
{
    int edge = pos[0] == e->N[0] - 1 || pos[1] == e->N[1] - 1 || pos[2] == e->N[2] - 1;
    for (int n = 0; n < 3; ++n) {
        int nP = (n + 1) % 3, nPP = (n + 2) % 3;
        unsigned ip[3] = {pos[0], pos[1], pos[2]};
        if (d->rho && d->interp == 0) {
            /* Operator_Cylinder::GetEdgeLength (FDTD/operator_cylinder.cpp:204-210): alpha edges
             * carry the rho of their line */
            double delta = (d->field == 0 ? d->el[n] : d->del[n])[ip[n]];
            if (n == 1)
                delta = delta * d->rho[ip[0]];
            double v = d->field == 0 ? (double)GETV(e, n, ip[0], ip[1], ip[2]) : (double)GETI(e, n, ip[0], ip[1], ip[2]);
            out[n] = delta != 0.0 ? v / delta : 0.0;
            continue;
        }
        if (d->field == 0) {
#define RAWE(p) (d->el[n][(p)[n]] ? (double)GETV(e, n, (p)[0], (p)[1], (p)[2]) / d->el[n][(p)[n]] : 0.0)
            if (d->interp == 0) {
                out[n] = RAWE(ip);
            } else if (d->interp == 1) {
                if (pos[n] == e->N[n] - 1) {
                    --ip[n];
                    out[n] = RAWE(ip);
                    continue;
                }
                double delta = d->el[n][ip[n]];
                out[n] = RAWE(ip);
                if (delta == 0) {
                    out[n] = 0;
                    continue;
                }
                if (pos[n] == 0)
                    continue;
                --ip[n];
                double deltaDown = d->el[n][ip[n]];
                double deltaRel = delta / (delta + deltaDown);
                out[n] = out[n] * (1.0 - deltaRel) + (double)RAWE(ip) * deltaRel;
            } else {
                if (edge) {
                    out[n] = 0;
                    continue;
                }
                out[n] = RAWE(ip);
                ++ip[nP];
                out[n] += RAWE(ip);
                ++ip[nPP];
                out[n] += RAWE(ip);
                --ip[nP];
                out[n] += RAWE(ip);
                out[n] /= 4;
            }
#undef RAWE
        } else {
#define RAWH(p) (d->del[n][(p)[n]] ? (double)GETI(e, n, (p)[0], (p)[1], (p)[2]) / d->del[n][(p)[n]] : 0.0)
            if (d->interp == 0) {
                out[n] = RAWH(ip);
            } else if (d->interp == 1) {
                if (edge || pos[nP] == 0 || pos[nPP] == 0) {
                    out[n] = 0;
                    continue;
                }
                out[n] = RAWH(ip);
                --ip[nP];
                out[n] += RAWH(ip);
                --ip[nPP];
                out[n] += RAWH(ip);
                ++ip[nP];
                out[n] += RAWH(ip);
                out[n] /= 4;
            } else {
                double delta = d->del[n][ip[n]];
                out[n] = RAWH(ip);
                if (pos[n] >= e->N[n] - 1) {
                    out[n] = 0;
                    continue;
                }
                ++ip[n];
                double deltaUp = d->del[n][ip[n]];
                double deltaRel = delta / (delta + deltaUp);
                out[n] = out[n] * (1.0 - deltaRel) + (double)RAWH(ip) * deltaRel;
            }
#undef RAWH
        }
    }
}

/* ProcessFieldsFD::Process (Common/processfields_fd.cpp:72-107) */
/* ProcessFieldsTD::Process (Common/processfields_td.cpp:50-91): ProcessFields::CalcField of the box
 * at a sample step, stored in float */
static void process_td(eng_t *e, dump_t *d)
{
    unsigned ts = e->numTS;
    if (ts < d->td_start || ts > d->td_stop || ts % d->td_interval)
        return;
    size_t plane = (size_t)d->sz[0] * d->sz[1] * d->sz[2];
    if (d->nsamp == d->cap) {
        d->cap = d->cap ? 2 * d->cap : 16;
        d->samp_ts = (unsigned *)realloc(d->samp_ts, (size_t)d->cap * 4);
        d->samples = (float *)realloc(d->samples, (size_t)d->cap * 3 * plane * 4);
        if (!d->samp_ts || !d->samples) {
            fprintf(stderr, "oracle: out of memory for time-domain samples\n");
            abort();
        }
    }
    float *out3 = d->samples + (size_t)d->nsamp * 3 * plane;
    size_t c = 0;
    unsigned pos[3];
    for (unsigned i = 0; i < d->sz[0]; ++i)
        for (unsigned j = 0; j < d->sz[1]; ++j)
            for (unsigned l = 0; l < d->sz[2]; ++l, ++c) {
                pos[0] = d->start[0] + i;
                pos[1] = d->start[1] + j;
                pos[2] = d->start[2] + l;
                double out[3];
                dump_field(e, d, pos, out);
                for (int n = 0; n < 3; ++n)
                    out3[(size_t)n * plane + c] = (float)out[n];
            }
    d->samp_ts[d->nsamp++] = ts;
}

static void process_dumps(eng_t *e)
{
    unsigned ts = e->numTS;
    for (int k = 0; k < e->ndumps; ++k) {
        dump_t *d = &e->dumps[k];
        if (d->td) {
            process_td(e, d);
            continue;
        }
        if (!d->fd_interval || ts % d->fd_interval)
            continue;
        double T = ((double)ts + (double)(d->field == 1) * 0.5) * e->dt;
        size_t plane = (size_t)d->sz[0] * d->sz[1] * d->sz[2];
        for (unsigned f = 0; f < d->nf; ++f) {
            float th = (float)(((-2.0 * M_PI_REF) * d->freqs[f]) * T);
            float complex ex = cexpf(CMPLXF(-0.0f, th));
            float er = crealf(ex) * 2.0f, ei = cimagf(ex) * 2.0f;
            float sc = (float)(e->dt * (double)d->fd_interval);
            er = er * sc;
            ei = ei * sc;
            float *acc = d->acc + (size_t)f * 3 * plane * 2;
            unsigned pos[3];
            size_t c = 0;
            for (unsigned i = 0; i < d->sz[0]; ++i)
                for (unsigned j = 0; j < d->sz[1]; ++j)
                    for (unsigned l = 0; l < d->sz[2]; ++l, ++c) {
                        pos[0] = d->start[0] + i;
                        pos[1] = d->start[1] + j;
                        pos[2] = d->start[2] + l;
                        double out[3];
                        dump_field(e, d, pos, out);
                        for (int n = 0; n < 3; ++n) {
                            float td = (float)out[n];
                            float *a = acc + ((size_t)n * plane + c) * 2;
                            a[0] = a[0] + td * er;
                            a[1] = a[1] + td * ei;
                        }
                    }
        }
    }
}

static void process_all(eng_t *e)
{
    process_probes(e);
    process_dumps(e);
}

/* ------------------------------------------------------------------------------------------ */
/* stepping */

/* Engine_Ext_Cylinder::DoPostVoltageUpdates (FDTD/extensions/engine_ext_cylinder.cpp:45-84):
 * the axis z voltage from the alpha currents around it, then the closed alpha seam */
static void cyl_post_volt(eng_t *e)
{
    if (!e->cyl_closed)
        return;
    const unsigned Nr = e->N[0], Na = e->N[1], Nz = e->N[2], last = Na - 2;
    if (e->cyl_r0) {
        for (unsigned z = 0; z < Nz; ++z) {
            float volt = GETV(e, 2, 0, 0, z) * e->cyl_vv_r0[z];
            for (unsigned a = 0; a < Na - 1; ++a)
                volt += e->cyl_vi_r0[z] * GETI(e, 1, 0, a, z);
            *fptr(e, 0, 2, 0, 0, z) = volt;
        }
        for (unsigned a = 0; a < Na; ++a)
            for (unsigned z = 0; z < Nz; ++z) {
                *fptr(e, 0, 1, 0, a, z) = 0;   /* no alpha voltage on the axis */
                *fptr(e, 0, 2, 0, a, z) = GETV(e, 2, 0, 0, z);
            }
    }
    for (unsigned r = 0; r < Nr; ++r)
        for (unsigned z = 0; z < Nz; ++z) {
            *fptr(e, 0, 0, r, 0, z) = GETV(e, 0, r, last, z);
            *fptr(e, 0, 2, r, 0, z) = GETV(e, 2, r, last, z);
        }
}

/* Engine_Ext_Cylinder::DoPostCurrentUpdates (:86-101): the tangential currents of alpha line 0
 * onto line N-2 */
static void cyl_post_curr(eng_t *e)
{
    if (!e->cyl_closed)
        return;
    const unsigned Nr = e->N[0], Na = e->N[1], Nz = e->N[2], last = Na - 2;
    for (unsigned r = 0; r + 1 < Nr; ++r)
        for (unsigned z = 0; z + 1 < Nz; ++z) {
            *fptr(e, 1, 0, r, last, z) = GETI(e, 0, r, 0, z);
            *fptr(e, 1, 2, r, last, z) = GETI(e, 2, r, 0, z);
        }
}

/* extension phases in reference order; thread 0 runs the non-threaded extensions */
static void pre_volt(eng_t *e)
{
    /* reverse priority: excitation (none), Mur walls (insertion order), Lorentz, UPML last */
    for (int w = 0; w < e->nmur; ++w)
        mur_pre(e, &e->mur[w]);
    for (int o = 0; o < e->nlor; ++o)
        lorentz_pre_volt(e, &e->lor[o]);
    rlc_pre(e);
}

static void post_volt_apply(eng_t *e)
{
    /* post hooks in priority order: UPML (run by the caller), cylinder (1e5), TFSF (5e4), Mur (0) */
    cyl_post_volt(e);
    tfsf_apply(e, 0);
    for (int w = e->nmur - 1; w >= 0; --w)
        mur_post(e, &e->mur[w]);
    /* apply hooks: lumped RLC (added last among the priority-0 extensions, so first after the
       reversed stable sort), dispersive, Mur, excitation */
    rlc_apply(e);
    for (int o = 0; o < e->nlor; ++o)
        lorentz_apply(e, &e->lor[o], 0);
    for (int w = e->nmur - 1; w >= 0; --w)
        mur_apply(e, &e->mur[w]);
    excitation_apply(e, 0);
}

static void pre_curr(eng_t *e)
{
    for (int o = 0; o < e->nlor; ++o)
        lorentz_pre_curr(e, &e->lor[o]);
}

static void post_curr_apply(eng_t *e)
{
    cyl_post_curr(e);
    tfsf_apply(e, 1);
    for (int o = 0; o < e->nlor; ++o)
        lorentz_apply(e, &e->lor[o], 1);
    excitation_apply(e, 1);
}

static void step_basic(eng_t *e)
{
    pre_volt(e);
    for (int r = e->nupml - 1; r >= 0; --r)
        upml_pre(e, &e->upml[r], 0, 0, e->upml[r].nl[0]);
    update_voltages_basic(e, 0, e->N[0]);
    for (int r = 0; r < e->nupml; ++r)
        upml_post(e, &e->upml[r], 0, 0, e->upml[r].nl[0]);
    post_volt_apply(e);

    pre_curr(e);
    for (int r = e->nupml - 1; r >= 0; --r)
        upml_pre(e, &e->upml[r], 1, 0, e->upml[r].nl[0]);
    update_currents_basic(e, 0, e->N[0] - 1);
    for (int r = 0; r < e->nupml; ++r)
        upml_post(e, &e->upml[r], 1, 0, e->upml[r].nl[0]);
    post_curr_apply(e);
    ++e->numTS;
}

/* x-slab split of a UPML region for thread tid (Engine_Ext_UPML::SetNumberOfThreads) */
static void upml_range(const eng_t *e, const upml_t *u, int tid, unsigned *x0, unsigned *x1)
{
    unsigned nt = (unsigned)e->nthreads, jobs = u->nl[0];
    unsigned base = jobs / nt, rem = jobs - base * nt, s = 0;
    for (int t = 0; t < tid; ++t)
        s += base + ((unsigned)t < rem);
    *x0 = s;
    *x1 = s + base + ((unsigned)tid < rem);
}

typedef struct {
    eng_t *e;
    int tid;
} targ_t;

static void *worker(void *arg)
{
    targ_t *ta = (targ_t *)arg;
    eng_t *e = ta->e;
    int tid = ta->tid;
    for (;;) {
        pthread_barrier_wait(&e->bar_start);
        if (e->stop_threads)
            break;
        for (unsigned it = 0; it < e->iter_ts; ++it) {
            unsigned x0, x1;
            if (tid == 0)
                pre_volt(e);
            pthread_barrier_wait(&e->bar_iter);
            for (int r = e->nupml - 1; r >= 0; --r) {
                upml_range(e, &e->upml[r], tid, &x0, &x1);
                upml_pre(e, &e->upml[r], 0, x0, x1);
                pthread_barrier_wait(&e->bar_iter);
            }
            update_voltages_mt(e, e->tstart[tid], e->tstop[tid] - e->tstart[tid] + 1);
            pthread_barrier_wait(&e->bar_iter);
            for (int r = 0; r < e->nupml; ++r) {
                upml_range(e, &e->upml[r], tid, &x0, &x1);
                upml_post(e, &e->upml[r], 0, x0, x1);
                pthread_barrier_wait(&e->bar_iter);
            }
            if (tid == 0)
                post_volt_apply(e);
            pthread_barrier_wait(&e->bar_iter);
            if (tid == 0)
                pre_curr(e);
            pthread_barrier_wait(&e->bar_iter);
            for (int r = e->nupml - 1; r >= 0; --r) {
                upml_range(e, &e->upml[r], tid, &x0, &x1);
                upml_pre(e, &e->upml[r], 1, x0, x1);
                pthread_barrier_wait(&e->bar_iter);
            }
            if (e->tstop_h[tid] + 1 > e->tstart[tid])
                update_currents_mt(e, e->tstart[tid], e->tstop_h[tid] - e->tstart[tid] + 1);
            pthread_barrier_wait(&e->bar_iter);
            for (int r = 0; r < e->nupml; ++r) {
                upml_range(e, &e->upml[r], tid, &x0, &x1);
                upml_post(e, &e->upml[r], 1, x0, x1);
                pthread_barrier_wait(&e->bar_iter);
            }
            if (tid == 0) {
                post_curr_apply(e);
                ++e->numTS;
                process_all(e);
            }
            pthread_barrier_wait(&e->bar_iter);
        }
        pthread_barrier_wait(&e->bar_stop);
    }
    free(ta);
    return NULL;
}

static int start_threads(eng_t *e)
{
    unsigned nt = (unsigned)e->nthreads;
    if (nt > e->N[0])
        nt = e->N[0];
    e->nthreads = (int)nt;
    /* Operator_Multithread::CalcStartStopLines (FDTD/operator_multithread.cpp:93-114) */
    e->tstart = (unsigned *)calloc(nt, 4);
    e->tstop = (unsigned *)calloc(nt, 4);
    e->tstop_h = (unsigned *)calloc(nt, 4);
    unsigned base = e->N[0] / nt, rem = e->N[0] - base * nt, s = 0;
    for (unsigned t = 0; t < nt; ++t) {
        unsigned jobs = base + (t < rem);
        e->tstart[t] = s;
        e->tstop[t] = s + jobs - 1;
        e->tstop_h[t] = (t == nt - 1) ? e->tstop[t] - 1 : e->tstop[t];
        s += jobs;
    }
    pthread_barrier_init(&e->bar_iter, NULL, nt);
    pthread_barrier_init(&e->bar_start, NULL, nt + 1);
    pthread_barrier_init(&e->bar_stop, NULL, nt + 1);
    e->threads = (pthread_t *)calloc(nt, sizeof(pthread_t));
    for (unsigned t = 0; t < nt; ++t) {
        targ_t *ta = (targ_t *)malloc(sizeof(targ_t));
        ta->e = e;
        ta->tid = (int)t;
        pthread_create(&e->threads[t], NULL, worker, ta);
    }
    return OK;
}

static void stop_threads(eng_t *e)
{
    e->stop_threads = 1;
    pthread_barrier_wait(&e->bar_start);
    for (int t = 0; t < e->nthreads; ++t)
        pthread_join(e->threads[t], NULL);
    free(e->threads);
    e->threads = NULL;
    pthread_barrier_destroy(&e->bar_iter);
    pthread_barrier_destroy(&e->bar_start);
    pthread_barrier_destroy(&e->bar_stop);
}

int oems_ref_init(eng_t *e, unsigned max_ts)
{
    if (!e || e->inited)
        return ERR_STATE;
    if (e->mt ? !e->op_index : !e->vv) {
        snprintf(e->err, sizeof e->err, "operator not set");
        return ERR_STATE;
    }
    e->maxTS = max_ts;
    for (int k = 0; k < e->nprobes; ++k) {
        probe_t *p = &e->probes[k];
        p->nslots = max_ts / p->interval + 1;
        p->series = (double *)malloc(p->nslots * p->ncomp * sizeof(double));
        for (size_t s = 0; s < p->nslots * p->ncomp; ++s)
            p->series[s] = NAN;
    }
    e->inited = 1;
    process_all(e);
    if (e->mt)
        return start_threads(e);
    return OK;
}

int oems_ref_iterate(eng_t *e, unsigned n)
{
    if (!e || !e->inited)
        return ERR_STATE;
    if (e->mt) {
        e->iter_ts = n;
        pthread_barrier_wait(&e->bar_start);
        pthread_barrier_wait(&e->bar_stop);
        return OK;
    }
    for (unsigned s = 0; s < n; ++s) {
        step_basic(e);
        process_all(e);
    }
    return OK;
}

int oems_ref_sync(eng_t *e)
{
    return e ? OK : ERR_ARG;
}

unsigned oems_ref_num_timesteps(const eng_t *e)
{
    return e ? e->numTS : 0;
}

/* ------------------------------------------------------------------------------------------ */
/* access */

int oems_ref_read_field(eng_t *e, int which, float *out)
{
    if (!e || !out || (which != 0 && which != 1))
        return ERR_ARG;
    if (!e->mt) {
        memcpy(out, which ? e->curr : e->volt, 3 * e->cells * sizeof(float));
        return OK;
    }
    for (unsigned n = 0; n < 3; ++n)
        for (unsigned x = 0; x < e->N[0]; ++x)
            for (unsigned y = 0; y < e->N[1]; ++y)
                for (unsigned z = 0; z < e->N[2]; ++z)
                    out[nijk(e, n, x, y, z)] = *fptr(e, which, n, x, y, z);
    return OK;
}

int oems_ref_write_field(eng_t *e, int which, const float *in)
{
    if (!e || !in || (which != 0 && which != 1))
        return ERR_ARG;
    for (unsigned n = 0; n < 3; ++n)
        for (unsigned x = 0; x < e->N[0]; ++x)
            for (unsigned y = 0; y < e->N[1]; ++y)
                for (unsigned z = 0; z < e->N[2]; ++z)
                    *fptr(e, which, n, x, y, z) = in[nijk(e, n, x, y, z)];
    return OK;
}

int oems_ref_get_value(eng_t *e, int which, unsigned n, unsigned x, unsigned y, unsigned z, float *v)
{
    if (!e || !v || n > 2 || x >= e->N[0] || y >= e->N[1] || z >= e->N[2])
        return ERR_ARG;
    *v = *fptr(e, which, n, x, y, z);
    return OK;
}

int oems_ref_set_value(eng_t *e, int which, unsigned n, unsigned x, unsigned y, unsigned z, float v)
{
    if (!e || n > 2 || x >= e->N[0] || y >= e->N[1] || z >= e->N[2])
        return ERR_ARG;
    *fptr(e, which, n, x, y, z) = v;
    return OK;
}

int oems_ref_read_probe(eng_t *e, int id, double *out, size_t cap, size_t *count)
{
    if (!e || id < 0 || id >= e->nprobes || !out || !count)
        return ERR_ARG;
    probe_t *p = &e->probes[id];
    size_t tot = p->nslots * p->ncomp;
    size_t n = tot < cap ? tot : cap;
    memcpy(out, p->series, n * sizeof(double));
    *count = n;
    return OK;
}

int oems_ref_read_probe_dft(eng_t *e, int id, double *out)
{
    if (!e || id < 0 || id >= e->nprobes || !out)
        return ERR_ARG;
    probe_t *p = &e->probes[id];
    memcpy(out, p->dft, 2 * p->nf * p->ncomp * sizeof(double));
    return OK;
}

int oems_ref_read_fd_dump(eng_t *e, int id, float *out, size_t cap)
{
    if (!e || id < 0 || id >= e->ndumps || !out)
        return ERR_ARG;
    dump_t *d = &e->dumps[id];
    size_t n = (size_t)d->nf * 3 * d->sz[0] * d->sz[1] * d->sz[2] * 2;
    if (cap < n)
        return ERR_ARG;
    memcpy(out, d->acc, n * sizeof(float));
    return OK;
}

/* Engine_Interface_FDTD::CalcFastEnergy (FDTD/engine_interface_fdtd.cpp:302-347) */
int oems_ref_energy(eng_t *e, double *out)
{
    if (!e || !out)
        return ERR_ARG;
    double E = 0.0, H = 0.0;
    for (unsigned x = 0; x + 1 < e->N[0]; ++x)
        for (unsigned y = 0; y + 1 < e->N[1]; ++y)
            for (unsigned z = 0; z + 1 < e->N[2]; ++z)
                for (int n = 0; n < 3; ++n) {
                    float v = GETV(e, n, x, y, z), c = GETI(e, n, x, y, z);
                    E += v * v;
                    H += c * c;
                }
    *out = EPS0 * E + MUE0 * H;
    return OK;
}
