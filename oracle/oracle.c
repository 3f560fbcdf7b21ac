/* oracle.c - CPU oracle: matrix-free PCG with a Jacobi or multigrid
 * preconditioner, restated in C from the reference's CPU solver.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): loaded by the tests, the smoke
 * check and the benchmark's CPU baseline leg, never by the product library.
 *
 * Build with -ffp-contract=off (oracle/Makefile does): the reference's results
 * depend on every rounding step, and a fused multiply-add changes them.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

#define R float
#define SFX _f
#include "oracle_mg.inc"
#undef R
#undef SFX

#define R double
#define SFX _d
#include "oracle_mg.inc"
#undef R
#undef SFX

/* Host copy of one level's operator and cell widths (MgLevelHost,
 * src/mg3d.h:88-93). */
typedef struct hlevel {
    int nx, ny, nz;
    double *dx, *dy;
    float *gE, *gN, *gU, *gB, *cap;
} hlevel;

struct oracle_solver {
    oracle_model m; /* fine operator (borrowed), P points at the copy below */
    int precond, mg_double, flexible;
    int outer_df;   /* outer vectors and updates in double-float (see below) */
    size_t n;
    double inv_dt;
    double *P, *x, *b, *r, *z, *p, *Ap, *invd;
    int nlev;
    hlevel* h;      /* operator of every level, finest first */
    level_f* lf;    /* float V-cycle state (mg_double == 0) */
    level_d* ld;    /* double V-cycle state (mg_double == 1) */
};

/* mg_coarse_cell (src/mg3d.h:100-136): sums in double in a fixed child order,
 * then one cast to float. */
static void coarse_cell(const hlevel* f, hlevel* c, int I, int J, int l) {
    const size_t fxy = (size_t)f->nx * f->ny, cxy = (size_t)c->nx * c->ny;
    const size_t cid = (size_t)l * cxy + (size_t)J * c->nx + I;
    const int i0 = 2 * I, i1 = (2 * I + 1 < f->nx - 1) ? 2 * I + 1 : f->nx - 1;
    const int j0 = 2 * J, j1 = (2 * J + 1 < f->ny - 1) ? 2 * J + 1 : f->ny - 1;
    double gu = 0, cp = 0, gb = 0;
    for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            const size_t fid = (size_t)l * fxy + (size_t)j * f->nx + i;
            gu += f->gU[fid];
            cp += f->cap[fid];
            if (l == 0) gb += f->gB[(size_t)j * f->nx + i];
        }
    c->gU[cid] = (float)gu;
    c->cap[cid] = (float)cp;
    if (l == 0) c->gB[(size_t)J * c->nx + I] = (float)gb;
    float e = 0.0f, nn = 0.0f;
    if (I < c->nx - 1) {
        double sum = 0;
        for (int j = j0; j <= j1; ++j) sum += f->gE[(size_t)l * fxy + (size_t)j * f->nx + 2 * I + 1];
        const double df = 0.5 * (f->dx[2 * I + 1] + f->dx[2 * I + 2]);
        const double dc = 0.5 * (c->dx[I] + c->dx[I + 1]);
        e = (float)(sum * df / dc);
    }
    if (J < c->ny - 1) {
        double sum = 0;
        for (int i = i0; i <= i1; ++i) sum += f->gN[(size_t)l * fxy + (size_t)(2 * J + 1) * f->nx + i];
        const double df = 0.5 * (f->dy[2 * J + 1] + f->dy[2 * J + 2]);
        const double dc = 0.5 * (c->dy[J] + c->dy[J + 1]);
        nn = (float)(sum * df / dc);
    }
    c->gE[cid] = e;
    c->gN[cid] = nn;
}

/* mg_coarse_widths (src/mg3d.h:139-144). */
static double* coarse_widths(const double* f, int n, int* cn) {
    *cn = (n + 1) / 2;
    double* c = (double*)malloc(sizeof(double) * (size_t)(*cn));
    for (int I = 0; I < *cn; ++I) c[I] = f[2 * I] + (2 * I + 1 < n ? f[2 * I + 1] : 0.0);
    return c;
}

static float* fdup(const float* v, size_t n) {
    float* o = (float*)malloc(sizeof(float) * n);
    memcpy(o, v, sizeof(float) * n);
    return o;
}

/* mg_build_levels (src/mg3d.h:147-183): finest first, down to 1 x 1. */
static hlevel* build_levels(const oracle_model* m, int* nlev_out) {
    int cap_lev = 64, nlev = 1;
    hlevel* L = (hlevel*)calloc((size_t)cap_lev, sizeof(hlevel));
    const size_t n = (size_t)m->nx * m->ny * m->nz, nxy = (size_t)m->nx * m->ny;
    L[0].nx = m->nx;
    L[0].ny = m->ny;
    L[0].nz = m->nz;
    L[0].dx = (double*)malloc(sizeof(double) * (size_t)m->nx);
    L[0].dy = (double*)malloc(sizeof(double) * (size_t)m->ny);
    for (int i = 0; i < m->nx; ++i) L[0].dx[i] = m->dx;
    for (int j = 0; j < m->ny; ++j) L[0].dy[j] = m->dy;
    L[0].gE = fdup(m->gE, n);
    L[0].gN = fdup(m->gN, n);
    L[0].gU = fdup(m->gU, n);
    L[0].gB = fdup(m->gB, nxy);
    L[0].cap = fdup(m->cap, n);
    while (L[nlev - 1].nx > 1 || L[nlev - 1].ny > 1) {
        const hlevel* f = &L[nlev - 1];
        hlevel c;
        c.nz = f->nz;
        c.dx = coarse_widths(f->dx, f->nx, &c.nx);
        c.dy = coarse_widths(f->dy, f->ny, &c.ny);
        const size_t cn = (size_t)c.nx * c.ny * c.nz, cxy = (size_t)c.nx * c.ny;
        c.gE = (float*)calloc(cn, sizeof(float));
        c.gN = (float*)calloc(cn, sizeof(float));
        c.gU = (float*)calloc(cn, sizeof(float));
        c.cap = (float*)calloc(cn, sizeof(float));
        c.gB = (float*)calloc(cxy, sizeof(float));
        for (int l = 0; l < c.nz; ++l)
            for (int J = 0; J < c.ny; ++J)
                for (int I = 0; I < c.nx; ++I) coarse_cell(f, &c, I, J, l);
        L[nlev++] = c;
    }
    *nlev_out = nlev;
    return L;
}

static oracle_model level_model(const hlevel* h) {
    oracle_model o;
    o.nx = h->nx;
    o.ny = h->ny;
    o.nz = h->nz;
    o.dx = 0;
    o.dy = 0;
    o.gE = h->gE;
    o.gN = h->gN;
    o.gU = h->gU;
    o.gB = h->gB;
    o.cap = h->cap;
    o.P = NULL;
    return o;
}

oracle_solver* oracle_create(const oracle_model* m, int precond, int mg_double, int flexible) {
    if (!m || m->nx < 1 || m->ny < 1 || m->nz < 1) return NULL;
    oracle_solver* s = (oracle_solver*)calloc(1, sizeof(oracle_solver));
    s->m = *m;
    s->precond = precond;
    s->mg_double = mg_double;
    s->flexible = flexible;
    s->n = (size_t)m->nx * m->ny * m->nz;
    double** vecs[] = {&s->P, &s->x, &s->b, &s->r, &s->z, &s->p, &s->Ap, &s->invd};
    for (size_t v = 0; v < sizeof(vecs) / sizeof(vecs[0]); ++v)
        *vecs[v] = (double*)calloc(s->n, sizeof(double));
    memcpy(s->P, m->P, sizeof(double) * s->n);
    s->m.P = s->P;
    if (precond == 1) {
        s->h = build_levels(m, &s->nlev);
        if (mg_double)
            s->ld = (level_d*)calloc((size_t)s->nlev, sizeof(level_d));
        else
            s->lf = (level_f*)calloc((size_t)s->nlev, sizeof(level_f));
        for (int k = 0; k < s->nlev; ++k) {
            const size_t ln = (size_t)s->h[k].nx * s->h[k].ny * s->h[k].nz;
            if (mg_double) {
                level_d* L = &s->ld[k];
                L->op = level_model(&s->h[k]);
                L->fcp = (double*)calloc(ln, sizeof(double));
                L->finv = (double*)calloc(ln, sizeof(double));
                L->x = (double*)calloc(ln, sizeof(double));
                L->b = (double*)calloc(ln, sizeof(double));
            } else {
                level_f* L = &s->lf[k];
                L->op = level_model(&s->h[k]);
                L->fcp = (float*)calloc(ln, sizeof(float));
                L->finv = (float*)calloc(ln, sizeof(float));
                L->x = (float*)calloc(ln, sizeof(float));
                L->b = (float*)calloc(ln, sizeof(float));
            }
        }
    }
    oracle_set_dt(s, 0.0);
    return s;
}

void oracle_destroy(oracle_solver* s) {
    if (!s) return;
    free(s->P); free(s->x); free(s->b); free(s->r); free(s->z); free(s->p); free(s->Ap);
    free(s->invd);
    for (int k = 0; k < s->nlev; ++k) {
        hlevel* h = &s->h[k];
        free(h->dx); free(h->dy); free(h->gE); free(h->gN); free(h->gU); free(h->gB);
        free(h->cap);
        if (s->ld) { free(s->ld[k].fcp); free(s->ld[k].finv); free(s->ld[k].x); free(s->ld[k].b); }
        if (s->lf) { free(s->lf[k].fcp); free(s->lf[k].finv); free(s->lf[k].x); free(s->lf[k].b); }
    }
    free(s->h);
    free(s->ld);
    free(s->lf);
    free(s);
}

/* CpuPcg::set_dt (src/pcg3d_cpu.cpp:41-57). */
void oracle_set_dt(oracle_solver* s, double dt) {
    s->inv_dt = dt > 0 ? 1.0 / dt : 0.0;
    const oracle_model* o = &s->m;
    for (int l = 0; l < o->nz; ++l)
        for (int j = 0; j < o->ny; ++j)
            for (int i = 0; i < o->nx; ++i) {
                const size_t id = ((size_t)l * o->ny + j) * o->nx + i;
                s->invd[id] = 1.0 / op_diag_d(o, i, j, l, s->inv_dt);
            }
    for (int k = 0; k < s->nlev; ++k) {
        if (s->mg_double) {
            level_d* L = &s->ld[k];
            for (int j = 0; j < L->op.ny; ++j)
                for (int i = 0; i < L->op.nx; ++i)
                    factor_column_d(&L->op, s->inv_dt, L->fcp, L->finv, i, j);
        } else {
            level_f* L = &s->lf[k];
            const float inv_dt = (float)s->inv_dt;
            for (int j = 0; j < L->op.ny; ++j)
                for (int i = 0; i < L->op.nx; ++i)
                    factor_column_f(&L->op, inv_dt, L->fcp, L->finv, i, j);
        }
    }
}

void oracle_set_x_zero(oracle_solver* s) { memset(s->x, 0, sizeof(double) * s->n); }
void oracle_set_x(oracle_solver* s, const double* x) { memcpy(s->x, x, sizeof(double) * s->n); }
void oracle_set_rhs_steady(oracle_solver* s) { memcpy(s->b, s->P, sizeof(double) * s->n); }
void oracle_set_power(oracle_solver* s, const double* P) { memcpy(s->P, P, sizeof(double) * s->n); }

/* CpuPcg::set_rhs_transient (src/pcg3d_cpu.cpp:63-65): b = P + C/dt x. */
void oracle_set_rhs_transient(oracle_solver* s) {
    for (size_t c = 0; c < s->n; ++c) s->b[c] = s->P[c] + (double)s->m.cap[c] * s->inv_dt * s->x[c];
}

void oracle_get_x(const oracle_solver* s, double* T) { memcpy(T, s->x, sizeof(double) * s->n); }

/* CpuPcg::precondition (src/pcg3d_cpu.cpp:115-124). */
static void precondition(oracle_solver* s) {
    if (s->precond == 0) {
        for (size_t c = 0; c < s->n; ++c) s->z[c] = s->r[c] * s->invd[c];
    } else if (s->mg_double) {
        level_d* L0 = &s->ld[0];
        for (size_t c = 0; c < s->n; ++c) L0->b[c] = s->r[c];
        vcycle_d(s->ld, s->nlev, 0, s->inv_dt);
        for (size_t c = 0; c < s->n; ++c) s->z[c] = L0->x[c];
    } else {
        level_f* L0 = &s->lf[0];
        for (size_t c = 0; c < s->n; ++c) L0->b[c] = (float)s->r[c];
        vcycle_f(s->lf, s->nlev, 0, (float)s->inv_dt);
        for (size_t c = 0; c < s->n; ++c) s->z[c] = (double)L0->x[c];
    }
}

static double dot(const double* a, const double* b, size_t n) {
    double s = 0;
    for (size_t c = 0; c < n; ++c) s += a[c] * b[c];
    return s;
}


/* ---- double-float outer iteration ------------------------------------------
 * An extension for the GPU library's FP32-pipe outer mode, not in the
 * reference: x, r, p, Ap and the diagonal are float pairs (hi + lo, about 48
 * significant bits) combined with error-free transformations (TwoSum,
 * Fast2Sum, FMA-based TwoProd, after Joldes, Muller and Popescu 2017), so that
 * the outer iteration runs on FP32 units; dots and alpha, beta are double. */
typedef struct dfl {
    float h, l;
} dfl;

static inline dfl df_two_sum(float a, float b) {
    const float s = a + b, bp = s - a, ap = s - bp;
    const float t = (a - ap) + (b - bp);
    dfl r = {s, t};
    return r;
}
static inline dfl df_fast(float a, float b) {
    const float s = a + b;
    dfl r = {s, b - (s - a)};
    return r;
}
static inline dfl df_of(double d) {
    const float h = (float)d;
    dfl r = {h, (float)(d - (double)h)};
    return r;
}
static inline double df_d(dfl x) { return (double)x.h + (double)x.l; }
static inline dfl df_add(dfl a, dfl b) {
    const dfl s = df_two_sum(a.h, b.h);
    return df_fast(s.h, s.l + (a.l + b.l));
}
static inline dfl df_neg(dfl a) {
    dfl r = {-a.h, -a.l};
    return r;
}
static inline dfl df_mul_f(dfl a, float b) {
    const float p = a.h * b;
    float e = fmaf(a.h, b, -p);
    e = fmaf(a.l, b, e);
    return df_fast(p, e);
}
static inline dfl df_mul(dfl a, dfl b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_fast(p, e);
}

void oracle_set_outer_df(oracle_solver* s, int on) { s->outer_df = on; }

/* Ap = d p - sum of G p_nbr with the diagonal in double-float. */
static void df_apply(const oracle_model* o, const dfl* dg, const dfl* p, dfl* Ap, double* pAp) {
    const size_t sxy = (size_t)o->nx * o->ny;
    double acc = 0;
    for (int l = 0; l < o->nz; ++l)
        for (int j = 0; j < o->ny; ++j)
            for (int i = 0; i < o->nx; ++i) {
                const size_t c = (size_t)l * sxy + (size_t)j * o->nx + i;
                dfl off = {0.0f, 0.0f};
                if (i > 0) off = df_add(off, df_mul_f(p[c - 1], o->gE[c - 1]));
                if (i < o->nx - 1) off = df_add(off, df_mul_f(p[c + 1], o->gE[c]));
                if (j > 0) off = df_add(off, df_mul_f(p[c - o->nx], o->gN[c - o->nx]));
                if (j < o->ny - 1) off = df_add(off, df_mul_f(p[c + o->nx], o->gN[c]));
                if (l > 0) off = df_add(off, df_mul_f(p[c - sxy], o->gU[c - sxy]));
                if (l < o->nz - 1) off = df_add(off, df_mul_f(p[c + sxy], o->gU[c]));
                Ap[c] = df_add(df_mul(dg[c], p[c]), df_neg(off));
                acc += df_d(p[c]) * df_d(Ap[c]);
            }
    *pAp = acc;
}

/* PCG with the outer iteration in double-float; same recurrence as
 * oracle_solve (flexible beta when s->flexible). */
static int solve_df(oracle_solver* s, double tol, int maxit, int* iters, double* relres) {
    const oracle_model* o = &s->m;
    const size_t n = s->n;
    for (int l = 0; l < o->nz; ++l)
        for (int j = 0; j < o->ny; ++j)
            for (int i = 0; i < o->nx; ++i) {
                const size_t c = ((size_t)l * o->ny + j) * o->nx + i;
                s->r[c] = s->b[c] - op_apply_d(o, s->x, i, j, l, s->inv_dt);
            }
    const double bb = dot(s->b, s->b, n);
    double rr = dot(s->r, s->r, n);
    *iters = 0;
    *relres = 0;
    if (bb == 0) {
        oracle_set_x_zero(s);
        return 1;
    }
    *relres = sqrt(rr / bb);
    if (*relres < tol) return 1;
    dfl* x = (dfl*)malloc(n * sizeof(dfl));
    dfl* r = (dfl*)malloc(n * sizeof(dfl));
    dfl* p = (dfl*)malloc(n * sizeof(dfl));
    dfl* Ap = (dfl*)malloc(n * sizeof(dfl));
    dfl* dg = (dfl*)malloc(n * sizeof(dfl));
    for (int l = 0; l < o->nz; ++l)
        for (int j = 0; j < o->ny; ++j)
            for (int i = 0; i < o->nx; ++i) {
                const size_t c = ((size_t)l * o->ny + j) * o->nx + i;
                dg[c] = df_of(op_diag_d(o, i, j, l, s->inv_dt));
            }
    for (size_t c = 0; c < n; ++c) {
        x[c] = df_of(s->x[c]);
        r[c] = df_of(s->r[c]);
    }
    int converged = 0;
    double rz = 0, pAp = 0;
    for (int it = 1; it <= maxit; ++it) {
        for (size_t c = 0; c < n; ++c) s->r[c] = r[c].h;  /* V-cycle input: float r */
        precondition(s);                                    /* z in s->z */
        double rz_new = 0, zAp = 0;
        for (size_t c = 0; c < n; ++c) {
            rz_new += df_d(r[c]) * s->z[c];
            zAp += s->z[c] * df_d(Ap[c]);
        }
        if (it == 1) {
            for (size_t c = 0; c < n; ++c) p[c] = df_of(s->z[c]);
        } else {
            const double beta = s->flexible ? -zAp / pAp : rz_new / rz;
            const dfl bdf = df_of(beta);
            for (size_t c = 0; c < n; ++c) p[c] = df_add(df_mul(bdf, p[c]), df_of(s->z[c]));
        }
        rz = rz_new;
        df_apply(o, dg, p, Ap, &pAp);
        const dfl a = df_of(rz / pAp);
        rr = 0;
        for (size_t c = 0; c < n; ++c) {
            x[c] = df_add(x[c], df_mul(a, p[c]));
            r[c] = df_add(r[c], df_neg(df_mul(a, Ap[c])));
            const double rv = df_d(r[c]);
            rr += rv * rv;
        }
        *iters = it;
        *relres = sqrt(rr / bb);
        if (*relres < tol) {
            converged = 1;
            break;
        }
    }
    for (size_t c = 0; c < n; ++c) s->x[c] = df_d(x[c]);
    free(x); free(r); free(p); free(Ap); free(dg);
    return converged;
}

/* CpuPcg::solve (src/pcg3d_cpu.cpp:126-185). */
int oracle_solve(oracle_solver* s, double tol, int maxit, int* iters, double* relres) {
    if (s->outer_df) return solve_df(s, tol, maxit, iters, relres);
    const oracle_model* o = &s->m;
    const size_t n = s->n;
    for (int l = 0; l < o->nz; ++l)
        for (int j = 0; j < o->ny; ++j)
            for (int i = 0; i < o->nx; ++i) {
                const size_t c = ((size_t)l * o->ny + j) * o->nx + i;
                s->r[c] = s->b[c] - op_apply_d(o, s->x, i, j, l, s->inv_dt);
            }
    const double bb = dot(s->b, s->b, n);
    double rr = dot(s->r, s->r, n);
    *iters = 0;
    *relres = 0;
    if (bb == 0) {
        oracle_set_x_zero(s);
        return 1;
    }
    *relres = sqrt(rr / bb);
    if (*relres < tol) return 1;

    precondition(s);
    memcpy(s->p, s->z, sizeof(double) * n);
    double rz = dot(s->r, s->z, n);
    int converged = 0;
    for (int it = 1; it <= maxit; ++it) {
        double pAp = 0;
        for (int l = 0; l < o->nz; ++l)
            for (int j = 0; j < o->ny; ++j)
                for (int i = 0; i < o->nx; ++i) {
                    const size_t c = ((size_t)l * o->ny + j) * o->nx + i;
                    s->Ap[c] = op_apply_d(o, s->p, i, j, l, s->inv_dt);
                    pAp += s->p[c] * s->Ap[c];
                }
        const double alpha = rz / pAp;
        rr = 0;
        for (size_t c = 0; c < n; ++c) {
            s->x[c] += alpha * s->p[c];
            s->r[c] -= alpha * s->Ap[c];
            rr += s->r[c] * s->r[c];
        }
        *iters = it;
        *relres = sqrt(rr / bb);
        if (*relres < tol) {
            converged = 1;
            break;
        }
        precondition(s);
        const double rz_new = dot(s->r, s->z, n);
        double beta;
        if (s->flexible)
            beta = -dot(s->z, s->Ap, n) / pAp;
        else
            beta = rz_new / rz;
        rz = rz_new;
        for (size_t c = 0; c < n; ++c) s->p[c] = s->z[c] + beta * s->p[c];
    }
    return converged;
}

int oracle_num_levels(const oracle_solver* s) { return s->nlev; }

void oracle_level_dims(const oracle_solver* s, int k, int* nx, int* ny, int* nz) {
    *nx = s->h[k].nx;
    *ny = s->h[k].ny;
    *nz = s->h[k].nz;
}

void oracle_level_operator(const oracle_solver* s, int k, float* gE, float* gN, float* gU,
                           float* gB, float* cap) {
    const hlevel* h = &s->h[k];
    const size_t n = (size_t)h->nx * h->ny * h->nz, nxy = (size_t)h->nx * h->ny;
    memcpy(gE, h->gE, n * sizeof(float));
    memcpy(gN, h->gN, n * sizeof(float));
    memcpy(gU, h->gU, n * sizeof(float));
    memcpy(gB, h->gB, nxy * sizeof(float));
    memcpy(cap, h->cap, n * sizeof(float));
}

void oracle_level_factors(const oracle_solver* s, int k, double* fcp, double* finv) {
    const hlevel* h = &s->h[k];
    const size_t n = (size_t)h->nx * h->ny * h->nz;
    for (size_t c = 0; c < n; ++c) {
        fcp[c] = s->mg_double ? s->ld[k].fcp[c] : (double)s->lf[k].fcp[c];
        finv[c] = s->mg_double ? s->ld[k].finv[c] : (double)s->lf[k].finv[c];
    }
}

/* true_relres (src/pcg3d_cpu.cpp:207-220). */
double oracle_true_relres(const oracle_model* m, const double* T) {
    double rr = 0, bb = 0;
    for (int l = 0; l < m->nz; ++l)
        for (int j = 0; j < m->ny; ++j)
            for (int i = 0; i < m->nx; ++i) {
                const size_t c = ((size_t)l * m->ny + j) * m->nx + i;
                const double r = m->P[c] - op_apply_d(m, T, i, j, l, 0.0);
                rr += r * r;
                bb += m->P[c] * m->P[c];
            }
    return sqrt(rr / bb);
}

void oracle_apply(const oracle_model* m, double inv_dt, const double* x, double* y) {
    for (int l = 0; l < m->nz; ++l)
        for (int j = 0; j < m->ny; ++j)
            for (int i = 0; i < m->nx; ++i)
                y[((size_t)l * m->ny + j) * m->nx + i] = op_apply_d(m, x, i, j, l, inv_dt);
}

/* heat_out (src/stack3d.h:252-263). */
double oracle_heat_out(const oracle_model* m, const double* T) {
    const size_t nxy = (size_t)m->nx * m->ny, top = (size_t)(m->nz - 1) * nxy;
    double q = 0;
    for (size_t c = 0; c < nxy; ++c) {
        q += (double)m->gU[top + c] * T[top + c];
        q += (double)m->gB[c] * T[c];
    }
    return q;
}

/* heat_stored (src/stack3d.h:265-273). */
double oracle_heat_stored(const oracle_model* m, const double* T_old, const double* T_new,
                          double dt) {
    const size_t n = (size_t)m->nx * m->ny * m->nz;
    double q = 0;
    for (size_t c = 0; c < n; ++c) q += (double)m->cap[c] * (T_new[c] - T_old[c]);
    return q / dt;
}

/* run_transient (src/transient3d.h:48-90). */
int oracle_run_transient(const oracle_model* m, int precond, int mg_double, int flexible,
                         double dt0, double growth, double dt_max, double t_end, int nsteps,
                         double tol, int maxit, double* rec, int max_rec, double* T_end,
                         long* total_iters, int* all_converged) {
    oracle_solver* s = oracle_create(m, precond, mg_double, flexible);
    if (!s) return -1;
    const size_t n = s->n;
    oracle_set_x_zero(s);
    double* T_old = (double*)calloc(n, sizeof(double));
    double* T_new = (double*)calloc(n, sizeof(double));
    double t = 0, dt = dt0, last_dt = -1;
    int steps = 0;
    long tot = 0;
    int allc = 1;
    while (nsteps > 0 ? steps < nsteps : t < t_end * (1 - 1e-12)) {
        if (nsteps <= 0 && t_end - t < dt) dt = t_end - t;
        if (dt != last_dt) {
            oracle_set_dt(s, dt);
            last_dt = dt;
        }
        oracle_set_rhs_transient(s);
        int it;
        double rel;
        const int conv = oracle_solve(s, tol, maxit, &it, &rel);
        oracle_get_x(s, T_new);
        t += dt;
        if (rec && steps < max_rec) {
            double tmax = T_new[0];
            for (size_t c = 1; c < n; ++c)
                if (T_new[c] > tmax) tmax = T_new[c];
            double* r = rec + 6 * (size_t)steps;
            r[0] = t;
            r[1] = dt;
            r[2] = it;
            r[3] = tmax;
            r[4] = oracle_heat_out(m, T_new);
            r[5] = oracle_heat_stored(m, T_old, T_new, dt);
        }
        tot += it;
        allc = allc && conv;
        double* tmp = T_old;
        T_old = T_new;
        T_new = tmp;
        dt = (dt_max < dt * growth) ? dt_max : dt * growth;
        ++steps;
    }
    if (T_end) memcpy(T_end, T_old, sizeof(double) * n);
    if (total_iters) *total_iters = tot;
    if (all_converged) *all_converged = allc;
    free(T_old);
    free(T_new);
    oracle_destroy(s);
    return steps;
}
