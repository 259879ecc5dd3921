/*
 * FP64 C oracle of the Fullwave 2.5 isotropic two-mechanism FDTD time loop (OpenMP).
 *
 * TEST INFRASTRUCTURE ONLY: a second, multi-threaded restatement of oracle/fdtd_oracle.py (same
 * scheme, same operation order, compiled with -ffp-contract=off) used by the tests as a faster
 * checker and by bench.py as the timed CPU baseline. The product never links it.
 *
 * Parity status: unpinned against the reference engine's output (closed x86-64 executables,
 * fullwave/solver/bins/gpu/{2d,3d}/num_relax=2/*, cannot run here or on the aarch64 GPU host);
 * its inputs are pinned to the reference's pre-processing by the golden fixtures.
 *
 * Scheme (see oracle/fdtd_oracle.py for the sources it follows):
 *   D_a f  = [sum_m c_m (f[+m e_a] - f[-(m-1) e_a]) + c_o sum_{b!=a, s=+-1} (f[e_a + s e_b] - f[s e_b])] / h_a
 *   psi    <- b_u psi + a_u D_a p ;  v_a <- v_a - dt/rho (D_a p / kappau + psi_1 + psi_2)
 *   D'_a g = [sum_m c_m (g[(m-1) e_a] - g[-m e_a]) + c_o sum (g[s e_b] - g[-e_a + s e_b])] / h_a
 *   phi    <- b_x phi + a_x D'_a v_a ;  p <- p - dt (K + 2 beta p) sum_a (D'_a v_a / kappax + phi_1 + phi_2)
 *   then p[icc] = icmat[:, n] (n < nTic), p[icczero] = 0, record p[outc] when n % modT == 0.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define GHOST 8

typedef struct {
    int ndim;
    int64_t n[3];       /* nx, ny, nz (nz = 1 in 2D) */
    double h[3], dt;
    int nt, nt_ic, mod_t, ncoords, ncoordsout, ncoordszero, ndmap;
    /* inputs (float32, dense C order) */
    const float *dmap;  /* [9][2][ndmap] */
    const int32_t *dcmap;
    const float *rho, *K, *beta;
    /* per derivative axis (the isotropic build passes the same maps for every axis):
       gradient maps kappa{u,w,v}, apml/bpml{u,w,v}{1,2}; divergence maps kappa{x,y,z}, ... */
    const float *kappau[3], *kappax[3];
    const float *au[3][2], *bu[3][2], *ax[3][2], *bx[3][2];
    const int32_t *icc, *outc, *icczero;
    const float *icmat; /* [ncoords][nt_ic] */
    const float *a_exp; /* non-NULL: exponential-attenuation engine (no memory variables) */
} oracle_desc;

typedef struct {
    oracle_desc d;
    int64_t cells, s[3];
    double *p, *v[3], *psi[3][2], *phi[3][2];
    double *taps;   /* per cell: 9 values */
    double *rdt_rho, *dtk, *b2dt, *iku[3], *ikx[3], *aexp;
    int has_beta;
    int64_t *icc_lin, *outc_lin, *zero_lin;
    int32_t *src_keep;
    int n_keep;
    int step;
} oracle_state;

static int64_t lin(const oracle_state *o, const int32_t *c) {
    int64_t idx = 0;
    for (int a = 0; a < o->d.ndim; ++a) idx += (int64_t)c[a] * o->s[a];
    return idx;
}

static int in_body(const oracle_state *o, int64_t c) {
    for (int a = 0; a < o->d.ndim; ++a) {
        int64_t q = (c / o->s[a]) % o->d.n[a];
        if (q < GHOST || q >= o->d.n[a] - GHOST) return 0;
    }
    return 1;
}

oracle_state *oracle_create(const oracle_desc *d) {
    oracle_state *o = calloc(1, sizeof(oracle_state));
    if (!o) return NULL;
    o->d = *d;
    if (d->ndim == 2) o->d.n[2] = 1;
    o->cells = o->d.n[0] * o->d.n[1] * o->d.n[2];
    o->s[2] = 1;
    o->s[1] = d->ndim == 3 ? o->d.n[2] : 1;
    o->s[0] = d->ndim == 3 ? o->d.n[1] * o->d.n[2] : o->d.n[1];
    const int64_t n = o->cells;
    double **fields[] = {&o->p, &o->v[0], &o->v[1], &o->v[2], &o->psi[0][0], &o->psi[0][1],
                         &o->psi[1][0], &o->psi[1][1], &o->psi[2][0], &o->psi[2][1],
                         &o->phi[0][0], &o->phi[0][1], &o->phi[1][0], &o->phi[1][1],
                         &o->phi[2][0], &o->phi[2][1], &o->rdt_rho, &o->dtk, &o->b2dt,
                         &o->iku[0], &o->iku[1], &o->iku[2], &o->ikx[0], &o->ikx[1], &o->ikx[2],
                         &o->aexp};
    for (size_t f = 0; f < sizeof fields / sizeof fields[0]; ++f) {
        *fields[f] = calloc((size_t)n, sizeof(double));
        if (!*fields[f]) return NULL;
    }
    o->taps = malloc((size_t)n * 9 * sizeof(double));
    for (int64_t c = 0; c < n; ++c) {
        int dc = d->dcmap[c];
        for (int m = 1; m <= 8; ++m) o->taps[c * 9 + m - 1] = (double)d->dmap[(m * 2 + 0) * d->ndmap + dc];
        o->taps[c * 9 + 8] = (double)d->dmap[(1 * 2 + 1) * d->ndmap + dc];
        o->rdt_rho[c] = d->dt / (double)d->rho[c];
        o->dtk[c] = d->dt * (double)d->K[c];
        o->b2dt[c] = 2.0 * d->dt * (double)d->beta[c];
        if (d->beta[c] != 0.f) o->has_beta = 1;
        if (d->a_exp) {
            o->aexp[c] = (double)d->a_exp[c];
            continue;
        }
        for (int a = 0; a < d->ndim; ++a) {
            o->iku[a][c] = 1.0 / (double)d->kappau[a][c];
            o->ikx[a][c] = 1.0 / (double)d->kappax[a][c];
        }
    }
    o->icc_lin = malloc(sizeof(int64_t) * (d->ncoords + 1));
    o->outc_lin = malloc(sizeof(int64_t) * (d->ncoordsout + 1));
    o->zero_lin = malloc(sizeof(int64_t) * (d->ncoordszero + 1));
    o->src_keep = malloc(sizeof(int32_t) * (d->ncoords + 1));
    for (int k = 0; k < d->ncoords; ++k) o->icc_lin[k] = lin(o, d->icc + (size_t)k * d->ndim);
    for (int k = 0; k < d->ncoordsout; ++k) o->outc_lin[k] = lin(o, d->outc + (size_t)k * d->ndim);
    for (int k = 0; k < d->ncoordszero; ++k) o->zero_lin[k] = lin(o, d->icczero + (size_t)k * d->ndim);
    /* the last listed source of a cell wins */
    o->n_keep = 0;
    for (int k = 0; k < d->ncoords; ++k) {
        int later = 0;
        for (int q = k + 1; q < d->ncoords && !later; ++q) later = o->icc_lin[q] == o->icc_lin[k];
        if (!later) o->src_keep[o->n_keep++] = k;
    }
    (void)in_body;
    return o;
}

void oracle_destroy(oracle_state *o) {
    if (!o) return;
    double *fields[] = {o->p, o->v[0], o->v[1], o->v[2], o->psi[0][0], o->psi[0][1],
                        o->psi[1][0], o->psi[1][1], o->psi[2][0], o->psi[2][1], o->phi[0][0],
                        o->phi[0][1], o->phi[1][0], o->phi[1][1], o->phi[2][0], o->phi[2][1],
                        o->rdt_rho, o->dtk, o->b2dt, o->iku[0], o->iku[1], o->iku[2],
                        o->ikx[0], o->ikx[1], o->ikx[2], o->aexp, o->taps};
    for (size_t f = 0; f < sizeof fields / sizeof fields[0]; ++f) free(fields[f]);
    free(o->icc_lin); free(o->outc_lin); free(o->zero_lin); free(o->src_keep);
    free(o);
}

#define BODY_LOOP(o, ...)                                                                    \
    _Pragma("omp parallel for collapse(2) schedule(static)")                                \
    for (int64_t i = GHOST; i < (o)->d.n[0] - GHOST; ++i)                                    \
        for (int64_t j = GHOST; j < (o)->d.n[1] - GHOST; ++j) {                             \
            const int64_t k0 = (o)->d.ndim == 3 ? GHOST : 0;                                \
            const int64_t k1 = (o)->d.ndim == 3 ? (o)->d.n[2] - GHOST : 1;                   \
            for (int64_t k = k0; k < k1; ++k) {                                              \
                const int64_t c = i * (o)->s[0] + j * (o)->s[1] + k;                           \
                __VA_ARGS__                                                                  \
            }                                                                                \
        }

static void step_exponential(oracle_state *o) {
    const int nd = o->d.ndim;
    for (int a = 0; a < nd; ++a) {
        const int64_t sa = o->s[a];
        const double h = o->d.h[a];
        double *p = o->p, *va = o->v[a];
        BODY_LOOP(o, {
            const double *t = o->taps + c * 9;
            double acc = 0.0, off = 0.0;
            for (int m = 1; m <= 8; ++m) acc += t[m - 1] * (p[c + m * sa] - p[c - (m - 1) * sa]);
            for (int b = 0; b < nd; ++b) {
                if (b == a) continue;
                const int64_t sb = o->s[b];
                off += p[c + sa + sb] - p[c + sb];
                off += p[c + sa - sb] - p[c - sb];
            }
            const double g = (acc + t[8] * off) / h;
            va[c] = o->aexp[c] * (va[c] - o->rdt_rho[c] * g);
        })
    }
    double *p = o->p;
    BODY_LOOP(o, {
        const double *t = o->taps + c * 9;
        double dsum = 0.0;
        for (int a = 0; a < nd; ++a) {
            const int64_t sa = o->s[a];
            const double *g = o->v[a];
            double acc = 0.0, off = 0.0;
            for (int m = 1; m <= 8; ++m) acc += t[m - 1] * (g[c + (m - 1) * sa] - g[c - m * sa]);
            for (int b = 0; b < nd; ++b) {
                if (b == a) continue;
                const int64_t sb = o->s[b];
                off += g[c + sb] - g[c - sa + sb];
                off += g[c - sb] - g[c - sa - sb];
            }
            dsum += (acc + t[8] * off) / o->d.h[a];
        }
        const double pb = p[c];
        const double coef = o->has_beta ? o->dtk[c] + o->b2dt[c] * pb : o->dtk[c];
        p[c] = o->aexp[c] * (pb - coef * dsum);
    })
}

void oracle_step(oracle_state *o, double *record_row) {
    const int nd = o->d.ndim;
    if (o->d.a_exp) {
        step_exponential(o);
        goto finish;
    }
    for (int a = 0; a < nd; ++a) {
        const int64_t sa = o->s[a];
        const double h = o->d.h[a];
        double *p = o->p, *va = o->v[a], *s1 = o->psi[a][0], *s2 = o->psi[a][1];
        BODY_LOOP(o, {
            const double *t = o->taps + c * 9;
            double acc = 0.0, off = 0.0;
            for (int m = 1; m <= 8; ++m) acc += t[m - 1] * (p[c + m * sa] - p[c - (m - 1) * sa]);
            for (int b = 0; b < nd; ++b) {
                if (b == a) continue;
                const int64_t sb = o->s[b];
                off += p[c + sa + sb] - p[c + sb];
                off += p[c + sa - sb] - p[c - sb];
            }
            const double g = (acc + t[8] * off) / h;
            s1[c] = o->d.bu[a][0][c] * s1[c] + o->d.au[a][0][c] * g;
            s2[c] = o->d.bu[a][1][c] * s2[c] + o->d.au[a][1][c] * g;
            va[c] -= o->rdt_rho[c] * (g * o->iku[a][c] + s1[c] + s2[c]);
        })
    }
    /* divergence accumulated per cell over axes in order, like the NumPy oracle */
    {
        double *p = o->p;
        BODY_LOOP(o, {
            const double *t = o->taps + c * 9;
            double dsum = 0.0;
            for (int a = 0; a < nd; ++a) {
                const int64_t sa = o->s[a];
                const double *g = o->v[a];
                double acc = 0.0, off = 0.0;
                for (int m = 1; m <= 8; ++m) acc += t[m - 1] * (g[c + (m - 1) * sa] - g[c - m * sa]);
                for (int b = 0; b < nd; ++b) {
                    if (b == a) continue;
                    const int64_t sb = o->s[b];
                    off += g[c + sb] - g[c - sa + sb];
                    off += g[c - sb] - g[c - sa - sb];
                }
                const double dv = (acc + t[8] * off) / o->d.h[a];
                double *f1 = o->phi[a][0], *f2 = o->phi[a][1];
                f1[c] = o->d.bx[a][0][c] * f1[c] + o->d.ax[a][0][c] * dv;
                f2[c] = o->d.bx[a][1][c] * f2[c] + o->d.ax[a][1][c] * dv;
                dsum += dv * o->ikx[a][c] + f1[c] + f2[c];
            }
            const double pb = p[c];
            if (o->has_beta) p[c] = pb - (o->dtk[c] + o->b2dt[c] * pb) * dsum;
            else p[c] = pb - o->dtk[c] * dsum;
        })
    }
finish:;
    const int n = o->step;
    if (n < o->d.nt_ic)
        for (int q = 0; q < o->n_keep; ++q) {
            const int k = o->src_keep[q];
            o->p[o->icc_lin[k]] = (double)o->d.icmat[(size_t)k * o->d.nt_ic + n];
        }
    for (int k = 0; k < o->d.ncoordszero; ++k) o->p[o->zero_lin[k]] = 0.0;
    if (record_row && n % o->d.mod_t == 0)
        for (int k = 0; k < o->d.ncoordsout; ++k) record_row[k] = o->p[o->outc_lin[k]];
    o->step++;
}

/* Run n_steps; traces [ceil(n_steps/mod_t)][ncoordsout] (FP64). */
void oracle_run(oracle_state *o, int n_steps, double *traces) {
    for (int s = 0; s < n_steps; ++s) {
        const int n = o->step;
        double *row = traces ? traces + (size_t)(n / o->d.mod_t) * o->d.ncoordsout : NULL;
        oracle_step(o, (n % o->d.mod_t == 0) ? row : NULL);
    }
}
