/*
 * sssi_oracle.c -- CPU restatement of SSSI's acoustic CPML finite-difference
 * hot path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and
 * the benchmark's CPU-baseline leg call it as the checker; the product never
 * links it.
 *
 * It restates, in plain C99 with every floating-point operation in the
 * reference's order (build with -ffp-contract=off so nothing is fused):
 *
 *   orc_dcoef        src/fd_cmex/finiteDifference.c:24-82 and src/dCoef.m:35-48
 *                    (A c = e1, A_ij = (2j-1)^(2i-1), solved by LU with partial
 *                    pivoting the way MATLAB's mldivide does)
 *   orc_damp_pml     src/fd_cmex/finiteDifference.c:253-280
 *   orc_fwd2d        src/fd_cmex/fwdTimeCpmlFor2dAw_mex.c:97-290
 *   orc_rvs2d        src/fd_cmex/rvsTimeCpmlFor2dAw_mex.c:86-287
 *   orc_fwd3d        src/fwdTimeCpmlFor3dAw.m:37-147 (MATLAB only in the
 *                    reference; cell-unit damping, velocity sampled from the
 *                    y=1 slice / top row as that file does)
 *   orc_image_accum  applications/rtm_2d_acoustic/mainRtmTimeCpmlFor2dAw.m:268-275
 *   orc_image_stack  applications/rtm_2d_acoustic/mainRtmTimeCpmlFor2dAw.m:315
 *   orc_diff_operator src/fd_cmex/diffOperator_mex.c:29-213 (the stand-alone
 *                    staggered derivative of a 2D/3D array along one dimension)
 *   orc_sponge2d     src/fwdTimeSpongeFor2dAw.m:36-101 and
 *                    src/rvsTimeSpongeFor2dAw.m:36-103 (MATLAB only in the
 *                    reference: second-order five-point update, sponge
 *                    factors on the new past and present)
 *
 * Index algebra of one step (0-based, column-major, l = 2N-1 zero rows and
 * columns of padding on every side of the padded wavefield P):
 *   D+ f(i) = sum_k (c_k*(f[i+1+k] - f[i-k]))/d      derivative at i+1/2
 *   D- g(i) = sum_k (c_k*(g[i+k]   - g[i-1-k]))/d    derivative at i from half points
 *   phi  = b*phi + (b-1)*D+P        (interior rows/columns only)
 *   A    = D+P + phi                (phi = 0 outside the interior)
 *   psi  = b*psi + (b-1)*D-A ;  Pz = D-A + psi
 *   Pnew = vdt^2*(Pz + Px + src) + 2*P - Pold
 * Each sum starts from 0.0 and adds the terms k = 0..N-1 in order.
 *
 * The loops are organised per column / per row (inner index contiguous) and
 * are OpenMP-parallel over the outer index; the arithmetic of every output
 * value is independent of that organisation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t idx_t;

static int omp_tid(void) {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

static int omp_nthreads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* stand-alone staggered derivative along dimension dim (1, 2 or 3) of an  */
/* n1 x n2 x n3 column-major array: out(m) = sum_k c_k (in(m+order+k) -   */
/* in(m+order-1-k)) / d, each term rounded separately, summed from 0 in    */
/* order of k; the output shrinks by 2 order - 1 along dim.               */
/* ------------------------------------------------------------------ */
void orc_diff_operator(const double *in, idx_t n1, idx_t n2, idx_t n3, const double *c, int order, double d,
                       int dim, double *out) {
    const idx_t l = 2 * (idx_t)order - 1;
    idx_t o1 = n1, o2 = n2, o3 = n3;
    if (dim == 1) o1 -= l;
    else if (dim == 2) o2 -= l;
    else o3 -= l;
    const idx_t s = dim == 1 ? 1 : (dim == 2 ? n1 : n1 * n2);
#pragma omp parallel for schedule(static)
    for (idx_t k = 0; k < o3; ++k)
        for (idx_t j = 0; j < o2; ++j)
            for (idx_t i = 0; i < o1; ++i) {
                const double *base = in + i + j * n1 + k * n1 * n2 + (idx_t)order * s;
                double acc = 0.0;
                for (int t = 0; t < order; ++t) {
                    const double diff = base[t * s] - base[-(t + 1) * s];
                    const double term = (c[t] * diff) / d;
                    acc = acc + term;
                }
                out[i + j * o1 + k * o1 * o2] = acc;
            }
}

/* ------------------------------------------------------------------ */
/* coefficients: LU with partial pivoting, reciprocal pivot scaling     */
/* ------------------------------------------------------------------ */
int orc_dcoef(int order, int staggered, double *coeff) {
    int n = order, i, j, k;
    double *A, *x;
    int *piv;
    if (n < 1 || n > 16) return 1;
    A = (double *)malloc(sizeof(double) * n * n);
    x = (double *)malloc(sizeof(double) * n);
    piv = (int *)malloc(sizeof(int) * n);
    for (j = 0; j < n; j++)
        for (i = 0; i < n; i++)
            A[i + j * n] = staggered ? pow(2 * (j + 1) - 1, 2 * (i + 1) - 1) : pow(j + 1, 2 * (i + 1) - 1);
    for (i = 0; i < n; i++) x[i] = 0.0;
    x[0] = staggered ? 1.0 : 0.5;

    for (k = 0; k < n; k++) {
        int p = k;
        double best = fabs(A[k + k * n]);
        for (i = k + 1; i < n; i++)
            if (fabs(A[i + k * n]) > best) {
                best = fabs(A[i + k * n]);
                p = i;
            }
        piv[k] = p;
        if (p != k)
            for (j = 0; j < n; j++) {
                double t = A[k + j * n];
                A[k + j * n] = A[p + j * n];
                A[p + j * n] = t;
            }
        if (A[k + k * n] != 0.0) {
            double r = 1.0 / A[k + k * n];
            for (i = k + 1; i < n; i++) A[i + k * n] *= r;
        }
        for (j = k + 1; j < n; j++) {
            double t = -A[k + j * n];
            for (i = k + 1; i < n; i++) A[i + j * n] += A[i + k * n] * t;
        }
    }
    for (k = 0; k < n; k++)
        if (piv[k] != k) {
            double t = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = t;
        }
    for (k = 0; k < n; k++)
        if (x[k] != 0.0)
            for (i = k + 1; i < n; i++) x[i] -= x[k] * A[i + k * n];
    for (k = n - 1; k >= 0; k--)
        if (x[k] != 0.0) {
            x[k] /= A[k + k * n];
            for (i = 0; i < k; i++) x[i] -= x[k] * A[i + k * n];
        }
    for (i = 0; i < n; i++) coeff[i] = x[i];
    free(A);
    free(x);
    free(piv);
    return 0;
}

/* d = (-(3 v)/(2 L) * log(R)) * (u/L) * (u/L), R = 1e-6 (C gateway order). */
void orc_damp_pml(const double *u, const double *v, idx_t count, double L, double *d) {
    const double logR = log(1e-6);
    idx_t q;
    for (q = 0; q < count; q++) {
        double d0 = -(3.0 * v[q]) / (2 * L) * logR;
        d[q] = d0 * (u[q] / L) * (u[q] / L);
    }
}

/* MATLAB dampPml.m order: d0 .* (u/L).^2 with .^2 an exact square. */
static double damp_matlab(double u, double v, double L) {
    const double logR = log(1e-6);
    double d0 = -(3 * v) / (2 * L) * logR;
    double q = u / L;
    return d0 * (q * q);
}

/*
 * 2D damping factors b = exp(-d dt) on the nz x nx grid (column-major),
 * with the conventions of fwdTimeCpmlFor2dAw_mex.c:100-145: left/right
 * u = (nB-j)*dx / (j+1)*dx, bottom u = (i+1)*dz, physical-unit L = nB*dx or
 * nB*dz, velocity of the damped cell itself, no top layer.
 */
void orc_damping_2d(const double *v, idx_t nz, idx_t nx, int nB, double dz, double dx, double dt, double *xb,
                    double *zb) {
    idx_t i, j;
    for (j = 0; j < nx; j++)
        for (i = 0; i < nz; i++) {
            double dxv = 0.0, dzv = 0.0;
            /* the right band is written after the left one in the reference,
             * so it wins where the two overlap */
            if (j >= nx - nB) {
                double u = (double)(j - (nx - nB) + 1) * dx;
                orc_damp_pml(&u, &v[i + j * nz], 1, nB * dx, &dxv);
            } else if (j < nB) {
                double u = (double)(nB - j) * dx;
                orc_damp_pml(&u, &v[i + j * nz], 1, nB * dx, &dxv);
            }
            if (i >= nz - nB) {
                double u = (double)(i - (nz - nB) + 1) * dz;
                orc_damp_pml(&u, &v[i + j * nz], 1, nB * dz, &dzv);
            }
            xb[i + j * nz] = exp(-dxv * dt);
            zb[i + j * nz] = exp(-dzv * dt);
        }
}

/* ------------------------------------------------------------------ */
/* one 2D step                                                          */
/* ------------------------------------------------------------------ */
typedef struct {
    idx_t nz, nx, Nz; /* Nz = nz + 2l: padded column length */
    int N, l;
    double dz, dx;
    const double *c;
    const double *xb, *zb, *vdt2; /* nz x nx */
    double *zphi, *zpsi;          /* nz x nx, interior rows only */
    double *xphi, *xpsi;          /* nz x nx, interior columns only */
    double *za;                   /* Nz x nx: zA for padded rows [N-1, Nz-N) */
    double *xa;                   /* nz x (nx+2l): xA for padded columns [N-1, Nx-N) */
    double *zp, *xp;              /* nz x nx */
    double *dtmp;                 /* one padded column of scratch per thread */
} step2d;

/* P: padded, Pn receives the new field (may alias nothing). src: value added at
 * interior (i,j) is src_dense[i + j*nz] if src_dense, else src_row[j] on i==0. */
static void step2d_run(step2d *s, const double *P, const double *Po, double *Pn, const double *src_dense,
                       const double *src_row) {
    const idx_t nz = s->nz, nx = s->nx, Nz = s->Nz;
    const int N = s->N, l = s->l;
    const double dz = s->dz, dx = s->dx;
    const double *c = s->c;
    idx_t j;

    /* z direction, one interior column at a time.  Each derivative is summed
     * over k in the outer loop so the inner loop over rows vectorises; every
     * element still sees the terms in the order k = 0..N-1. */
#pragma omp parallel for schedule(static)
    for (j = 0; j < nx; j++) {
        const double *Pc = P + (j + l) * Nz;
        double *za = s->za + j * Nz;
        double *dcol = s->dtmp + (idx_t)omp_tid() * Nz;
        idx_t i;
        int k;
        for (i = N - 1; i < Nz - N; i++) dcol[i] = 0.0;
        for (k = 0; k < N; k++) {
            const double ck = c[k];
            for (i = N - 1; i < Nz - N; i++) dcol[i] = dcol[i] + ck * (Pc[i + 1 + k] - Pc[i - k]) / dz;
        }
        for (i = N - 1; i < l; i++) za[i] = dcol[i] + 0.0;
        for (i = l; i < nz + l; i++) {
            idx_t q = (i - l) + j * nz;
            s->zphi[q] = s->zb[q] * s->zphi[q] + (s->zb[q] - 1) * dcol[i];
            za[i] = dcol[i] + s->zphi[q];
        }
        for (i = nz + l; i < Nz - N; i++) za[i] = dcol[i] + 0.0;
        for (i = l; i < nz + l; i++) dcol[i] = 0.0;
        for (k = 0; k < N; k++) {
            const double ck = c[k];
            for (i = l; i < nz + l; i++) dcol[i] = dcol[i] + ck * (za[i + k] - za[i - 1 - k]) / dz;
        }
        for (i = l; i < nz + l; i++) {
            idx_t q = (i - l) + j * nz;
            s->zpsi[q] = s->zb[q] * s->zpsi[q] + (s->zb[q] - 1) * dcol[i];
            s->zp[q] = dcol[i] + s->zpsi[q];
        }
    }

    /* x direction: xA over padded columns [N-1, nx+2l-N), rows interior */
#pragma omp parallel for schedule(static)
    for (j = N - 1; j < nx + 2 * l - N; j++) {
        double *xa = s->xa + j * nz;
        double *dcol = s->dtmp + (idx_t)omp_tid() * Nz;
        idx_t i;
        int k;
        for (i = 0; i < nz; i++) dcol[i] = 0.0;
        for (k = 0; k < N; k++) {
            const double ck = c[k];
            const double *pa = P + l + (j + 1 + k) * Nz, *pb = P + l + (j - k) * Nz;
            for (i = 0; i < nz; i++) dcol[i] = dcol[i] + ck * (pa[i] - pb[i]) / dx;
        }
        if (j >= l && j < nx + l) {
            for (i = 0; i < nz; i++) {
                idx_t q = i + (j - l) * nz;
                s->xphi[q] = s->xb[q] * s->xphi[q] + (s->xb[q] - 1) * dcol[i];
                xa[i] = dcol[i] + s->xphi[q];
            }
        } else {
            for (i = 0; i < nz; i++) xa[i] = dcol[i] + 0.0;
        }
    }
#pragma omp parallel for schedule(static)
    for (j = l; j < nx + l; j++) {
        double *dcol = s->dtmp + (idx_t)omp_tid() * Nz;
        idx_t i;
        int k;
        for (i = 0; i < nz; i++) dcol[i] = 0.0;
        for (k = 0; k < N; k++) {
            const double ck = c[k];
            const double *xa_p = s->xa + (j + k) * nz, *xa_m = s->xa + (j - 1 - k) * nz;
            for (i = 0; i < nz; i++) dcol[i] = dcol[i] + ck * (xa_p[i] - xa_m[i]) / dx;
        }
        for (i = 0; i < nz; i++) {
            idx_t q = i + (j - l) * nz;
            s->xpsi[q] = s->xb[q] * s->xpsi[q] + (s->xb[q] - 1) * dcol[i];
            s->xp[q] = dcol[i] + s->xpsi[q];
        }
    }

    /* update */
#pragma omp parallel for schedule(static)
    for (j = 0; j < nx; j++) {
        idx_t i;
        for (i = 0; i < nz; i++) {
            idx_t q = i + j * nz, p = (i + l) + (j + l) * Nz;
            double sv = src_dense ? src_dense[q] : ((src_row && i == 0) ? src_row[j] : 0.0);
            Pn[p] = s->vdt2[q] * (s->zp[q] + s->xp[q] + sv) + 2 * P[p] - Po[p];
        }
    }
}

static int step2d_init(step2d *s, const double *v, idx_t nz, idx_t nx, int N, int nB, double dz, double dx, double dt,
                       double *coeff) {
    idx_t q, n = nz * nx;
    memset(s, 0, sizeof(*s));
    s->nz = nz;
    s->nx = nx;
    s->N = N;
    s->l = 2 * N - 1;
    s->Nz = nz + 2 * s->l;
    s->dz = dz;
    s->dx = dx;
    if (orc_dcoef(N, 1, coeff)) return 1;
    s->c = coeff;
    s->xb = (double *)malloc(sizeof(double) * n);
    s->zb = (double *)malloc(sizeof(double) * n);
    s->vdt2 = (double *)malloc(sizeof(double) * n);
    orc_damping_2d(v, nz, nx, nB, dz, dx, dt, (double *)s->xb, (double *)s->zb);
    for (q = 0; q < n; q++) ((double *)s->vdt2)[q] = (v[q] * dt) * (v[q] * dt);
    s->zphi = (double *)calloc(n, sizeof(double));
    s->zpsi = (double *)calloc(n, sizeof(double));
    s->xphi = (double *)calloc(n, sizeof(double));
    s->xpsi = (double *)calloc(n, sizeof(double));
    s->zp = (double *)calloc(n, sizeof(double));
    s->xp = (double *)calloc(n, sizeof(double));
    s->za = (double *)calloc(s->Nz * nx, sizeof(double));
    s->xa = (double *)calloc(nz * (nx + 2 * s->l), sizeof(double));
    s->dtmp = (double *)calloc(s->Nz * (idx_t)omp_nthreads(), sizeof(double));
    return 0;
}

static void step2d_free(step2d *s) {
    free((void *)s->xb);
    free((void *)s->zb);
    free((void *)s->vdt2);
    free(s->zphi);
    free(s->zpsi);
    free(s->xphi);
    free(s->xpsi);
    free(s->zp);
    free(s->xp);
    free(s->za);
    free(s->xa);
    free(s->dtmp);
}

static void copy_interior(const double *P, idx_t nz, idx_t nx, idx_t Nz, int l, double *out) {
    idx_t j;
    for (j = 0; j < nx; j++) memcpy(out + j * nz, P + l + (j + l) * Nz, sizeof(double) * nz);
}

/*
 * Forward modelling (fwdTimeCpmlFor2dAw_mex).  v: nz x nx; source: nz x nx x nt
 * (column-major) or NULL with (src_trace, src_iz, src_ix) for one point
 * source whose amplitude at step t is src_trace[t]; data: nx x nt (or NULL);
 * snapshot: nz x nx x nt (or NULL); t_count limits the number of steps run
 * (t_count <= nt, used for bounded timing samples).
 */
int orc_fwd2d(const double *v, const double *source, const double *src_trace, idx_t src_iz, idx_t src_ix, idx_t nz,
              idx_t nx, idx_t nt, int N, int nB, double dz, double dx, double dt, double *data, double *snapshot) {
    step2d s;
    double coeff[16];
    idx_t t, Np;
    double *Pa, *Pb, *Pc;
    double *slice = NULL;
    if (step2d_init(&s, v, nz, nx, N, nB, dz, dx, dt, coeff)) return 1;
    Np = s.Nz * (nx + 2 * s.l);
    Pa = (double *)calloc(Np, sizeof(double)); /* old */
    Pb = (double *)calloc(Np, sizeof(double)); /* cur */
    Pc = (double *)calloc(Np, sizeof(double)); /* new */
    if (!source && src_trace) slice = (double *)calloc(nz * nx, sizeof(double));
    for (t = 0; t < nt; t++) {
        const double *src = source ? source + t * nz * nx : NULL;
        double *tmp;
        if (slice) {
            slice[src_iz + src_ix * nz] = src_trace[t];
            src = slice;
        }
        step2d_run(&s, Pb, Pa, Pc, src, NULL);
        tmp = Pa; /* old <- cur, cur <- new */
        Pa = Pb;
        Pb = Pc;
        Pc = tmp;
        if (data) {
            idx_t j;
            for (j = 0; j < nx; j++) data[j + t * nx] = Pb[s.l + (j + s.l) * s.Nz];
        }
        if (snapshot) copy_interior(Pb, nz, nx, s.Nz, s.l, snapshot + t * nz * nx);
    }
    free(Pa);
    free(Pb);
    free(Pc);
    free(slice);
    step2d_free(&s);
    return 0;
}

/*
 * Reverse propagation (rvsTimeCpmlFor2dAw_mex).  data: nx x nt injected on
 * interior row 0, time running nt-1 .. 0.  model receives the padded field
 * (nz+2l) x (nx+2l) held as "old" after the loop, i.e. the field produced by
 * the step before the last one (rvsTimeCpmlFor2dAw_mex.c:262,285-287).
 * If fwd_snap is given (nz x nx x nt forward snapshots), the imaging sums
 * img_m += f_t .* r_t and img_s2 += f_t.^2 are accumulated as each reverse
 * snapshot r_t is produced (t descending).
 */
int orc_rvs2d(const double *v, const double *data, idx_t nz, idx_t nx, idx_t nt, int N, int nB, double dz, double dx,
              double dt, double *model, double *snapshot, const double *fwd_snap, double *img_m, double *img_s2) {
    step2d s;
    double coeff[16];
    idx_t t, Np;
    double *Pa, *Pb, *Pc;
    if (step2d_init(&s, v, nz, nx, N, nB, dz, dx, dt, coeff)) return 1;
    Np = s.Nz * (nx + 2 * s.l);
    Pa = (double *)calloc(Np, sizeof(double));
    Pb = (double *)calloc(Np, sizeof(double));
    Pc = (double *)calloc(Np, sizeof(double));
    for (t = nt - 1; t >= 0; t--) {
        double *tmp;
        step2d_run(&s, Pb, Pa, Pc, NULL, data + t * nx);
        tmp = Pa;
        Pa = Pb;
        Pb = Pc;
        Pc = tmp;
        if (snapshot) copy_interior(Pb, nz, nx, s.Nz, s.l, snapshot + t * nz * nx);
        if (fwd_snap && img_m && img_s2) {
            idx_t i, j;
            const double *f = fwd_snap + t * nz * nx;
            for (j = 0; j < nx; j++)
                for (i = 0; i < nz; i++) {
                    idx_t q = i + j * nz;
                    double r = Pb[(i + s.l) + (j + s.l) * s.Nz];
                    img_m[q] = f[q] * r + img_m[q];
                    img_s2[q] = f[q] * f[q] + img_s2[q];
                }
        }
    }
    if (model) memcpy(model, Pa, sizeof(double) * Np);
    free(Pa);
    free(Pb);
    free(Pc);
    step2d_free(&s);
    return 0;
}

/* M = f.*r + M ; s2 = f.^2 + s2 over one snapshot pair (n cells). */
void orc_image_accum(const double *f, const double *r, idx_t n, double *m, double *s2) {
    idx_t q;
    for (q = 0; q < n; q++) {
        m[q] = f[q] * r[q] + m[q];
        s2[q] = f[q] * f[q] + s2[q];
    }
}

/* Stacked = Stacked + M ./ s2 */
void orc_image_stack(const double *m, const double *s2, idx_t n, double *stacked) {
    idx_t q;
    for (q = 0; q < n; q++) stacked[q] = stacked[q] + m[q] / s2[q];
}

/* ------------------------------------------------------------------ */
/* 3D forward (fwdTimeCpmlFor3dAw.m)                                    */
/* ------------------------------------------------------------------ */
/*
 * Damping of the 3D MATLAB file: u and L in cells (L = nB), x profiles from
 * the y=1 slice v(:, ixb, 1) replicated along y, y profiles from the top row
 * v(1, :, iyb) replicated along z, z profiles from v(izb2, :, 1) replicated
 * along y (fwdTimeCpmlFor3dAw.m:53-70).
 */
void orc_damping_3d(const double *v, idx_t nz, idx_t nx, idx_t ny, int nB, double dt, double *xb, double *yb,
                    double *zb) {
    idx_t i, j, k;
    const idx_t sxy = nz * nx;
    for (k = 0; k < ny; k++)
        for (j = 0; j < nx; j++)
            for (i = 0; i < nz; i++) {
                double dxv = 0.0, dyv = 0.0, dzv = 0.0;
                idx_t q = i + j * nz + k * sxy;
                if (j < nB)
                    dxv = damp_matlab((double)(nB - j), v[i + j * nz], (double)nB);
                else if (j >= nx - nB)
                    dxv = damp_matlab((double)(j - (nx - nB) + 1), v[i + j * nz], (double)nB);
                if (k < nB)
                    dyv = damp_matlab((double)(nB - k), v[j * nz + k * sxy], (double)nB);
                else if (k >= ny - nB)
                    dyv = damp_matlab((double)(k - (ny - nB) + 1), v[j * nz + k * sxy], (double)nB);
                if (i >= nz - nB) dzv = damp_matlab((double)(i - (nz - nB) + 1), v[i + j * nz], (double)nB);
                xb[q] = exp(-dxv * dt);
                yb[q] = exp(-dyv * dt);
                zb[q] = exp(-dzv * dt);
            }
}

/*
 * v: nz x nx x ny; source: nz x nx x ny x nt, or NULL with one point source
 * (src_trace, src_iz, src_ix, src_iy).  data: nx x ny x nt (top interior
 * face) or NULL; snapshot: nz x nx x ny x nt or NULL.
 */
int orc_fwd3d(const double *v, const double *source, const double *src_trace, idx_t src_iz, idx_t src_ix,
              idx_t src_iy, idx_t nz, idx_t nx, idx_t ny, idx_t nt, int N, int nB, double dz, double dx, double dy,
              double dt, double *data, double *snapshot) {
    const int l = 2 * N - 1;
    const idx_t Nz = nz + 2 * l, Nx = nx + 2 * l, Ny = ny + 2 * l;
    const idx_t n = nz * nx * ny, Np = Nz * Nx * Ny;
    const idx_t sP = Nz * Nx; /* padded plane stride */
    const idx_t sI = nz * nx; /* interior plane stride */
    double c[16];
    double *xb, *yb, *zb, *vdt2, *zphi, *xphi, *yphi, *zpsi, *xpsi, *ypsi, *zp, *xp, *yp, *za, *xa, *ya;
    double *Pa, *Pb, *Pc, *slice = NULL;
    idx_t q, t;
    if (orc_dcoef(N, 1, c)) return 1;
    xb = (double *)malloc(sizeof(double) * n);
    yb = (double *)malloc(sizeof(double) * n);
    zb = (double *)malloc(sizeof(double) * n);
    vdt2 = (double *)malloc(sizeof(double) * n);
    orc_damping_3d(v, nz, nx, ny, nB, dt, xb, yb, zb);
    for (q = 0; q < n; q++) vdt2[q] = (v[q] * dt) * (v[q] * dt);
    zphi = (double *)calloc(n, sizeof(double));
    xphi = (double *)calloc(n, sizeof(double));
    yphi = (double *)calloc(n, sizeof(double));
    zpsi = (double *)calloc(n, sizeof(double));
    xpsi = (double *)calloc(n, sizeof(double));
    ypsi = (double *)calloc(n, sizeof(double));
    zp = (double *)calloc(n, sizeof(double));
    xp = (double *)calloc(n, sizeof(double));
    yp = (double *)calloc(n, sizeof(double));
    za = (double *)calloc(Nz * nx * ny, sizeof(double));
    xa = (double *)calloc(nz * Nx * ny, sizeof(double));
    ya = (double *)calloc(nz * nx * Ny, sizeof(double));
    Pa = (double *)calloc(Np, sizeof(double));
    Pb = (double *)calloc(Np, sizeof(double));
    Pc = (double *)calloc(Np, sizeof(double));
    if (!source && src_trace) slice = (double *)calloc(n, sizeof(double));

#define PIDX(i, j, k) ((i) + (j) * Nz + (k) * sP)
    for (t = 0; t < nt; t++) {
        const double *src = source ? source + t * n : NULL;
        double *tmp;
        idx_t k;
        if (slice) {
            slice[src_iz + src_ix * nz + src_iy * sI] = src_trace[t];
            src = slice;
        }
        /* z */
#pragma omp parallel for schedule(static)
        for (k = 0; k < ny; k++) {
            idx_t i, j;
            int m;
            for (j = 0; j < nx; j++) {
                const double *Pcol = Pb + PIDX(0, j + l, k + l);
                double *zac = za + j * Nz + k * Nz * nx;
                for (i = N - 1; i < Nz - N; i++) {
                    double d = 0.0;
                    for (m = 0; m < N; m++) d = d + c[m] * (Pcol[i + 1 + m] - Pcol[i - m]) / dz;
                    if (i >= l && i < nz + l) {
                        idx_t qq = (i - l) + j * nz + k * sI;
                        zphi[qq] = zb[qq] * zphi[qq] + (zb[qq] - 1) * d;
                        zac[i] = d + zphi[qq];
                    } else {
                        zac[i] = d + 0.0;
                    }
                }
                for (i = l; i < nz + l; i++) {
                    idx_t qq = (i - l) + j * nz + k * sI;
                    double d = 0.0;
                    for (m = 0; m < N; m++) d = d + c[m] * (zac[i + m] - zac[i - 1 - m]) / dz;
                    zpsi[qq] = zb[qq] * zpsi[qq] + (zb[qq] - 1) * d;
                    zp[qq] = d + zpsi[qq];
                }
            }
        }
        /* x */
#pragma omp parallel for schedule(static)
        for (k = 0; k < ny; k++) {
            idx_t i, j;
            int m;
            for (j = N - 1; j < Nx - N; j++) {
                double *xac = xa + j * nz + k * nz * Nx;
                for (i = 0; i < nz; i++) {
                    double d = 0.0;
                    for (m = 0; m < N; m++)
                        d = d + c[m] * (Pb[PIDX(i + l, j + 1 + m, k + l)] - Pb[PIDX(i + l, j - m, k + l)]) / dx;
                    if (j >= l && j < nx + l) {
                        idx_t qq = i + (j - l) * nz + k * sI;
                        xphi[qq] = xb[qq] * xphi[qq] + (xb[qq] - 1) * d;
                        xac[i] = d + xphi[qq];
                    } else {
                        xac[i] = d + 0.0;
                    }
                }
            }
            for (j = l; j < nx + l; j++) {
                for (i = 0; i < nz; i++) {
                    idx_t qq = i + (j - l) * nz + k * sI;
                    const double *xk = xa + k * nz * Nx;
                    double d = 0.0;
                    for (m = 0; m < N; m++) d = d + c[m] * (xk[i + (j + m) * nz] - xk[i + (j - 1 - m) * nz]) / dx;
                    xpsi[qq] = xb[qq] * xpsi[qq] + (xb[qq] - 1) * d;
                    xp[qq] = d + xpsi[qq];
                }
            }
        }
        /* y */
#pragma omp parallel for schedule(static)
        for (k = N - 1; k < Ny - N; k++) {
            idx_t i, j;
            int m;
            for (j = 0; j < nx; j++)
                for (i = 0; i < nz; i++) {
                    double d = 0.0;
                    for (m = 0; m < N; m++)
                        d = d + c[m] * (Pb[PIDX(i + l, j + l, k + 1 + m)] - Pb[PIDX(i + l, j + l, k - m)]) / dy;
                    if (k >= l && k < ny + l) {
                        idx_t qq = i + j * nz + (k - l) * sI;
                        yphi[qq] = yb[qq] * yphi[qq] + (yb[qq] - 1) * d;
                        ya[i + j * nz + k * sI] = d + yphi[qq];
                    } else {
                        ya[i + j * nz + k * sI] = d + 0.0;
                    }
                }
        }
#pragma omp parallel for schedule(static)
        for (k = l; k < ny + l; k++) {
            idx_t i, j;
            int m;
            for (j = 0; j < nx; j++)
                for (i = 0; i < nz; i++) {
                    idx_t qq = i + j * nz + (k - l) * sI;
                    double d = 0.0;
                    for (m = 0; m < N; m++)
                        d = d + c[m] * (ya[i + j * nz + (k + m) * sI] - ya[i + j * nz + (k - 1 - m) * sI]) / dy;
                    ypsi[qq] = yb[qq] * ypsi[qq] + (yb[qq] - 1) * d;
                    yp[qq] = d + ypsi[qq];
                }
        }
        /* update */
#pragma omp parallel for schedule(static)
        for (k = 0; k < ny; k++) {
            idx_t i, j;
            for (j = 0; j < nx; j++)
                for (i = 0; i < nz; i++) {
                    idx_t qq = i + j * nz + k * sI, p = PIDX(i + l, j + l, k + l);
                    double sv = src ? src[qq] : 0.0;
                    Pc[p] = vdt2[qq] * (zp[qq] + xp[qq] + yp[qq] + sv) + 2 * Pb[p] - Pa[p];
                }
        }
        tmp = Pa;
        Pa = Pb;
        Pb = Pc;
        Pc = tmp;
        if (data) {
            idx_t j;
            for (k = 0; k < ny; k++)
                for (j = 0; j < nx; j++) data[j + k * nx + t * nx * ny] = Pb[PIDX(l, j + l, k + l)];
        }
        if (snapshot) {
            idx_t j;
            for (k = 0; k < ny; k++)
                for (j = 0; j < nx; j++)
                    memcpy(snapshot + t * n + j * nz + k * sI, Pb + PIDX(l, j + l, k + l), sizeof(double) * nz);
        }
    }
#undef PIDX
    free(xb);
    free(yb);
    free(zb);
    free(vdt2);
    free(zphi);
    free(xphi);
    free(yphi);
    free(zpsi);
    free(xpsi);
    free(ypsi);
    free(zp);
    free(xp);
    free(yp);
    free(za);
    free(xa);
    free(ya);
    free(Pa);
    free(Pb);
    free(Pc);
    free(slice);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Sponge-ABC propagation (forward, or reverse with data on row 0).  The    */
/* zero-bordered (nz+2) x (nx+2) fields of the MATLAB file, its expression */
/* order b.*P - Pold + ax.*(R+L) + az.*(D+U) - vdtSq.*src, the rotation     */
/* and the sponge loop over ixb = 2..nB+1 (left column, right column,       */
/* bottom row; past then present) as written.  src_dense: nz x nx x nt;     */
/* point sources: nsrc cells with wavelets[k*nt + t]; rdata (reverse): nx x  */
/* nt on row 0.  Outputs (each optional): data nx x nt, snapshot nz x nx x  */
/* nt, last (nz x nx, the present after the final step).                   */
/* ------------------------------------------------------------------ */
int orc_sponge2d(const double *v, idx_t nz, idx_t nx, idx_t nt, int nB, double dz, double dx, double dt,
                 const double *src_dense, int nsrc, const idx_t *src_iz, const idx_t *src_ix, const double *wav,
                 const double *rdata, double *data, double *snapshot, double *last) {
    const idx_t Nz = nz + 2, Nx = nx + 2, n = nz * nx;
    double *bnd = (double *)malloc(sizeof(double) * (nB > 0 ? nB : 1));
    double *ax = (double *)malloc(sizeof(double) * n), *az = (double *)malloc(sizeof(double) * n);
    double *vs = (double *)malloc(sizeof(double) * n), *b = (double *)malloc(sizeof(double) * n);
    double *f1 = (double *)calloc((size_t)(Nz * Nx), sizeof(double));
    double *f2 = (double *)calloc((size_t)(Nz * Nx), sizeof(double));
    double *f3 = (double *)calloc((size_t)(Nz * Nx), sizeof(double));
    double *src = (double *)calloc((size_t)n, sizeof(double));
    if (!bnd || !ax || !az || !vs || !b || !f1 || !f2 || !f3 || !src) return -1;
    for (int iz = 0; iz < nB; ++iz) {
        const double a = 0.015 * (double)(nB - iz);
        bnd[iz] = pow(exp(-(a * a)), 10.0);
    }
    for (idx_t q = 0; q < n; ++q) {
        double t = v[q] * dt / dx;
        ax[q] = t * t;
        t = v[q] * dt / dz;
        az[q] = t * t;
        t = v[q] * dt;
        vs[q] = t * t;
        b[q] = 2 - 2 * ax[q] - 2 * az[q];
    }
    for (idx_t step = 0; step < nt; ++step) {
        const idx_t it = rdata ? nt - 1 - step : step;
        const double *sl = NULL;
        if (src_dense) {
            sl = src_dense + it * n;
        } else if (nsrc > 0 || rdata) {
            memset(src, 0, sizeof(double) * n);
            if (rdata)
                for (idx_t j = 0; j < nx; ++j) src[j * nz] = rdata[j + it * nx];
            for (int k = 0; k < nsrc; ++k) {
                const idx_t q = src_iz[k] + src_ix[k] * nz;
                int dup = 0;
                for (int m = 0; m < k; ++m) dup |= src_iz[m] == src_iz[k] && src_ix[m] == src_ix[k];
                src[q] = dup ? src[q] + wav[k * nt + it] : wav[k * nt + it];
            }
            sl = src;
        }
#pragma omp parallel for schedule(static)
        for (idx_t j = 0; j < nx; ++j)
            for (idx_t i = 0; i < nz; ++i) {
                const idx_t p = (i + 1) + (j + 1) * Nz, q = i + j * nz;
                double r = b[q] * f2[p] - f1[p] + ax[q] * (f2[p + Nz] + f2[p - Nz]) + az[q] * (f2[p + 1] + f2[p - 1]);
                if (sl) r = r - vs[q] * sl[q];
                f3[p] = r;
            }
        double *tmp = f1; /* fdm1 <- fdm2, fdm2 <- fdm3 (f3 is fully rewritten next step) */
        f1 = f2;
        f2 = f3;
        f3 = tmp;
        for (int ixb = 2; ixb <= nB + 1; ++ixb) {
            const idx_t c = ixb - 1, c2 = nx - nB + ixb - 1, r2 = nz - nB + ixb - 1;
            const double bl = bnd[ixb - 2], br = bnd[nx - (nx - nB + ixb) + 1], bb = bnd[nz - (nz - nB + ixb) + 1];
            double *fs[2] = {f1, f2};
            for (int w = 0; w < 2; ++w)
                for (idx_t i = 1; i <= nz - nB; ++i) fs[w][i + c * Nz] = bl * fs[w][i + c * Nz];
            for (int w = 0; w < 2; ++w)
                for (idx_t i = 1; i <= nz - nB; ++i) fs[w][i + c2 * Nz] = br * fs[w][i + c2 * Nz];
            for (int w = 0; w < 2; ++w)
                for (idx_t j = 0; j < Nx; ++j) fs[w][r2 + j * Nz] = bb * fs[w][r2 + j * Nz];
        }
        if (data)
            for (idx_t j = 0; j < nx; ++j) data[j + it * nx] = f2[1 + (j + 1) * Nz];
        if (snapshot)
            for (idx_t j = 0; j < nx; ++j)
                memcpy(snapshot + it * n + j * nz, f2 + 1 + (j + 1) * Nz, sizeof(double) * nz);
    }
    if (last)
        for (idx_t j = 0; j < nx; ++j) memcpy(last + j * nz, f2 + 1 + (j + 1) * Nz, sizeof(double) * nz);
    free(bnd);
    free(ax);
    free(az);
    free(vs);
    free(b);
    free(f1);
    free(f2);
    free(f3);
    free(src);
    return 0;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
