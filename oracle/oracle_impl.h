/*
 * Precision-generic body of the CPU oracle.  Included twice by
 * acumen_oracle.c: once with REAL=float (the reference's own single
 * precision, evaluated in source order with no contraction) and once with
 * REAL=double (the FP64 oracle).  TEST INFRASTRUCTURE ONLY: the product path
 * never links this code.
 *
 * Array conventions follow the reference's Fortran column-major storage:
 *   image  img(jx,jy)       -> img[(jy-1)*N + (jx-1)]          (x fastest)
 *   sino   sino(jbin,jtheta)-> sino[(jtheta-1)*N + (jbin-1)]   (bin fastest)
 * and S slices are stored one after another.
 */

#ifndef REAL
#error "REAL must be defined"
#endif

/* floor() of a coordinate as an int, without a libm call: truncate, then
 * step down for negative non-integers.  Equal to (int)floor(x) wherever the
 * result fits an int, which every grid coordinate here does.              */
static inline int SFX(ifloor)(REAL x)
{
    int i = (int)x;
    return i - ((REAL)i > x);
}

/* tomography/tv_hpc.F90:53-56 -- filter taps, jx = 1..2N+1 */
void SFX(orc_filter_taps)(int N, REAL *filt)
{
    const REAL pi = R(4.0) * RATAN(R(1.0));
    for (int jx = 1; jx <= 2 * N + 1; ++jx) {
        long k = (long)(jx - 1 - N);
        long den = 4 * k * k - 1;                 /* integer arithmetic */
        filt[jx - 1] = -((R(2.0) * (REAL)N) / ((pi * pi) * (REAL)den));
    }
}

/* tomography/tv_hpc.F90:58-74 -- circular mask with exp taper, times pi/T */
void SFX(orc_cmask)(int N, int T, int wpu, REAL *cmask)
{
    const REAL pi = R(4.0) * RATAN(R(1.0));
    const REAL rad_n = (REAL)(N - 1) / R(2.0) - (REAL)wpu;
    for (int jy = 1; jy <= N; ++jy) {
        for (int jx = 1; jx <= N; ++jx) {
            REAL ax = ((REAL)jx - ((REAL)N - R(1.0)) / R(2.0)) - R(1.0);
            REAL ay = ((REAL)jy - ((REAL)N - R(1.0)) / R(2.0)) - R(1.0);
            REAL rr = RSQRT(ax * ax + ay * ay);
            REAL rtmp = R(1.0) - (R(2.0) * (rr - rad_n)) / (REAL)wpu;
            REAL v;
            if (rtmp <= R(0.0)) {
                v = R(0.0);
            } else if (rtmp >= R(1.0)) {
                v = pi / (REAL)T;
            } else {
                REAL in = RE(R(1.0) - R(1.0) / (R(1.0) - rtmp));
                v = (pi * RE(R(1.0) - R(1.0) / (R(1.0) - in))) / (REAL)T;
            }
            cmask[(size_t)(jy - 1) * N + (jx - 1)] = v;
        }
    }
}

/* Per-angle (sin, cos) of the two angle conventions used by the reference:
 *   backprojection  ctheta = pi*(90-theta)/180   (tv_hpc.F90:113)
 *   projector       ctheta = pi*(theta-90)/180   (tv_hpc.F90:142)            */
static void SFX(angle_tables)(int T, const float *theta, REAL *sb, REAL *cb,
                              REAL *sf, REAL *cf)
{
    const REAL pi = R(4.0) * RATAN(R(1.0));
    for (int t = 0; t < T; ++t) {
        REAL th = (REAL)theta[t];
        REAL ctb = (pi * (R(90.0) - th)) / R(180.0);
        REAL ctf = (pi * (th - R(90.0))) / R(180.0);
        if (sb) sb[t] = RSIN(ctb);
        if (cb) cb[t] = RCOS(ctb);
        if (sf) sf[t] = RSIN(ctf);
        if (cf) cf[t] = RCOS(ctf);
    }
}

/* tomography/tv_hpc.F90:93-105 -- direct "same" convolution of every column */
void SFX(orc_filter)(int N, int T, int S, const REAL *sino, REAL *out)
{
    REAL *filt = (REAL *)malloc(sizeof(REAL) * (size_t)(2 * N + 1));
    SFX(orc_filter_taps)(N, filt);
    const int nfilt = 2 * N + 1, nstart = N;
    long rows = (long)S * T;
#pragma omp parallel for schedule(static)
    for (long row = 0; row < rows; ++row) {
        const REAL *x = sino + (size_t)row * N;
        REAL *y = out + (size_t)row * N;
        for (int jy = 1; jy <= N; ++jy) {
            REAL sum = R(0.0);
            for (int jx = 1; jx <= N; ++jx) {
                int jk = jy - jx + 1 + nstart;
                if (jk > 1 && jk < nfilt + 1) sum = sum + x[jx - 1] * filt[jk - 1];
            }
            y[jy - 1] = sum;
        }
    }
    free(filt);
}

/* tomography/tv_hpc.F90:107-123 -- pixel-driven linear-interpolation
 * backprojection of an already filtered sinogram, times cmask.            */
void SFX(orc_backproject)(int N, int T, const float *theta, int wpu, int S,
                          const REAL *sinoCS, REAL *img)
{
    REAL *sb = (REAL *)malloc(sizeof(REAL) * T), *cb = (REAL *)malloc(sizeof(REAL) * T);
    REAL *cmask = (REAL *)malloc(sizeof(REAL) * (size_t)N * N);
    SFX(angle_tables)(T, theta, sb, cb, NULL, NULL);
    SFX(orc_cmask)(N, T, wpu, cmask);
    const REAL mid = (REAL)((N + 1) / 2);       /* integer division, tv_hpc.F90:15 */
    long rows = (long)S * N;
#pragma omp parallel for schedule(static)
    for (long row = 0; row < rows; ++row) {
        int s = (int)(row / N), jy = (int)(row % N) + 1;
        const REAL *q = sinoCS + (size_t)s * T * N;
        REAL *o = img + (size_t)s * N * N + (size_t)(jy - 1) * N;
        for (int jx = 1; jx <= N; ++jx) {
            REAL sum = R(0.0);
            for (int t = 0; t < T; ++t) {
                REAL yr = (sb[t] * ((REAL)jx - mid) + cb[t] * ((REAL)jy - mid)) + mid;
                int y1 = SFX(ifloor)(yr);
                int y2 = y1 + 1;
                if (y1 > 1 && y2 < N + 1) {
                    const REAL *qt = q + (size_t)t * N;
                    sum = (sum + qt[y1 - 1] * ((REAL)y2 - yr)) + qt[y2 - 1] * (yr - (REAL)y1);
                }
            }
            o[jx - 1] = cmask[(size_t)(jy - 1) * N + (jx - 1)] * sum;
        }
    }
    free(sb); free(cb); free(cmask);
}

/* tomography/tv_hpc.F90:84-126 -- iradon = filter + backprojection + mask */
void SFX(orc_iradon)(int N, int T, const float *theta, int wpu, int S,
                     const REAL *sino, REAL *img)
{
    REAL *cs = (REAL *)malloc(sizeof(REAL) * (size_t)S * T * N);
    SFX(orc_filter)(N, T, S, sino, cs);
    SFX(orc_backproject)(N, T, theta, wpu, S, cs, img);
    free(cs);
}

/* tomography/tv_hpc.F90:129-159 -- bilinear ray-sum projector, divided by N */
void SFX(orc_radon)(int N, int T, const float *theta, int S, const REAL *img, REAL *sino)
{
    REAL *sf = (REAL *)malloc(sizeof(REAL) * T), *cf = (REAL *)malloc(sizeof(REAL) * T);
    SFX(angle_tables)(T, theta, NULL, NULL, sf, cf);
    const REAL mid = (REAL)((N + 1) / 2);
    long rows = (long)S * T;
#pragma omp parallel for schedule(static)
    for (long row = 0; row < rows; ++row) {
        int s = (int)(row / T), t = (int)(row % T);
        const REAL *u = img + (size_t)s * N * N;
        REAL *o = sino + (size_t)s * T * N + (size_t)t * N;
        const REAL c = cf[t], sn = sf[t];
        for (int jy = 1; jy <= N; ++jy) {
            REAL sum = R(0.0);
            for (int jx = 1; jx <= N; ++jx) {
                REAL xr = (c * ((REAL)jx - mid) - sn * ((REAL)jy - mid)) + mid;
                REAL yr = (sn * ((REAL)jx - mid) + c * ((REAL)jy - mid)) + mid;
                int y1 = SFX(ifloor)(yr), y2 = y1 + 1;
                int x1 = SFX(ifloor)(xr), x2 = x1 + 1;
                int mn = x1 < y1 ? x1 : y1, mx = x2 > y2 ? x2 : y2;
                if (mn > 1 && mx < N + 1) {
                    REAL a = u[(size_t)(y1 - 1) * N + (x1 - 1)];
                    REAL b = u[(size_t)(y1 - 1) * N + (x2 - 1)];
                    REAL cc = u[(size_t)(y2 - 1) * N + (x1 - 1)];
                    REAL d = u[(size_t)(y2 - 1) * N + (x2 - 1)];
                    REAL wxl = (REAL)x2 - xr, wxh = xr - (REAL)x1;
                    REAL wyl = (REAL)y2 - yr, wyh = yr - (REAL)y1;
                    sum = (((sum + (a * wxl) * wyl) + (b * wxh) * wyl) + (cc * wxl) * wyh) + (d * wxh) * wyh;
                }
            }
            o[jy - 1] = sum / (REAL)N;
        }
    }
    free(sf); free(cf);
}

/* Exact transpose of orc_radon (not in the reference): every projector sample
 * scatters y(jbin,theta)/N times its four bilinear weights back into the
 * taps it read.  Summation order: theta, bin, step (sequential).           */
void SFX(orc_radon_adjoint)(int N, int T, const float *theta, int S, const REAL *sino, REAL *img)
{
    REAL *sf = (REAL *)malloc(sizeof(REAL) * T), *cf = (REAL *)malloc(sizeof(REAL) * T);
    SFX(angle_tables)(T, theta, NULL, NULL, sf, cf);
    const REAL mid = (REAL)((N + 1) / 2);
#pragma omp parallel for schedule(dynamic)
    for (int s = 0; s < S; ++s) {
        REAL *u = img + (size_t)s * N * N;
        memset(u, 0, sizeof(REAL) * (size_t)N * N);
        for (int t = 0; t < T; ++t) {
            const REAL c = cf[t], sn = sf[t];
            const REAL *yv = sino + (size_t)s * T * N + (size_t)t * N;
            for (int jy = 1; jy <= N; ++jy) {
                REAL w = yv[jy - 1] / (REAL)N;
                for (int jx = 1; jx <= N; ++jx) {
                    REAL xr = (c * ((REAL)jx - mid) - sn * ((REAL)jy - mid)) + mid;
                    REAL yr = (sn * ((REAL)jx - mid) + c * ((REAL)jy - mid)) + mid;
                    int y1 = SFX(ifloor)(yr), y2 = y1 + 1;
                    int x1 = SFX(ifloor)(xr), x2 = x1 + 1;
                    int mn = x1 < y1 ? x1 : y1, mx = x2 > y2 ? x2 : y2;
                    if (mn > 1 && mx < N + 1) {
                        REAL wxl = (REAL)x2 - xr, wxh = xr - (REAL)x1;
                        REAL wyl = (REAL)y2 - yr, wyh = yr - (REAL)y1;
                        u[(size_t)(y1 - 1) * N + (x1 - 1)] += (w * wxl) * wyl;
                        u[(size_t)(y1 - 1) * N + (x2 - 1)] += (w * wxh) * wyl;
                        u[(size_t)(y2 - 1) * N + (x1 - 1)] += (w * wxl) * wyh;
                        u[(size_t)(y2 - 1) * N + (x2 - 1)] += (w * wxh) * wyh;
                    }
                }
            }
        }
    }
    free(sf); free(cf);
}

/* Periodic neighbour indices of tomography/tv_hpc.F90:220-237 (1-based). */
static inline int SFX(nb_next)(int j, int N) { return j + 1 - ((j + 1) / (N + 1)) * N; }
static inline int SFX(nb_prev)(int j, int N) { return j - 1 + N - ((j - 1 + N) / (N + 1)) * N; }

/* Reductions: red_mode 0 = the reference's single-precision running sum in
 * loop order (jy outer, jx inner); red_mode 1 = the same order accumulated in
 * double.  The FP64 instantiation always accumulates in double.            */
static double SFX(sum_sq)(int N, const REAL *a, int red_mode)
{
    if (red_mode == 0 && sizeof(REAL) == sizeof(float)) {
        float s = 0.0f;
        for (size_t i = 0; i < (size_t)N * N; ++i) s = s + (float)a[i] * (float)a[i];
        return s;
    }
    double s = 0.0;
    for (size_t i = 0; i < (size_t)N * N; ++i) s += (double)a[i] * (double)a[i];
    return s;
}
static double SFX(sum_dot)(int N, const REAL *a, const REAL *b, int red_mode)
{
    if (red_mode == 0 && sizeof(REAL) == sizeof(float)) {
        float s = 0.0f;
        for (size_t i = 0; i < (size_t)N * N; ++i) s = s + (float)a[i] * (float)b[i];
        return s;
    }
    double s = 0.0;
    for (size_t i = 0; i < (size_t)N * N; ++i) s += (double)a[i] * (double)b[i];
    return s;
}

/* tomography/tv_hpc.F90:253-300 -- one CG step of the inner solve on
 * M = mu*iradon(radon(.)) + lambda*(periodic Laplacian): rp = radon(p),
 * irpt = iradon(rp), Ap, alpha = rsold/<p,Ap>, uk += alpha p, r -= alpha Ap,
 * beta = rsnew/rsold, p = r + beta p.  Returns rsnew.  Work arrays: Ap, irpt
 * (N*N) and rp (N*T).                                                       */
double SFX(orc_cg_step)(int N, int T, const float *theta, int wpu, REAL lambda, REAL mu, int red_mode,
                        REAL *uk, REAL *r, REAL *p, REAL *Ap, REAL *rp, REAL *irpt, double rsold)
{
    size_t NN = (size_t)N * N;
#define AT(a, x, y) (a)[(size_t)((y) - 1) * N + ((x) - 1)]
    SFX(orc_radon)(N, T, theta, 1, p, rp);
    SFX(orc_iradon)(N, T, theta, wpu, 1, rp, irpt);
    for (int jy = 1; jy <= N; ++jy)
        for (int jx = 1; jx <= N; ++jx) {
            int jxr = SFX(nb_next)(jx, N), jyr = SFX(nb_next)(jy, N);
            int jxl = SFX(nb_prev)(jx, N), jyl = SFX(nb_prev)(jy, N);
            REAL lap = (((R(4.0) * AT(p, jx, jy) - AT(p, jxl, jy)) - AT(p, jxr, jy)) - AT(p, jx, jyl)) - AT(p, jx, jyr);
            AT(Ap, jx, jy) = mu * AT(irpt, jx, jy) + lambda * lap;
        }
#undef AT
    double num = SFX(sum_dot)(N, p, Ap, red_mode);
    REAL alpha;
    if (red_mode == 0 && sizeof(REAL) == sizeof(float)) alpha = (REAL)((float)rsold / (float)num);
    else alpha = (REAL)(rsold / num);
    for (size_t i = 0; i < NN; ++i) {
        uk[i] = uk[i] + alpha * p[i];
        r[i] = r[i] - alpha * Ap[i];
    }
    double rsnew = SFX(sum_sq)(N, r, red_mode);
    REAL beta;
    if (red_mode == 0 && sizeof(REAL) == sizeof(float)) beta = (REAL)((float)rsnew / (float)rsold);
    else beta = (REAL)(rsnew / rsold);
    for (size_t i = 0; i < NN; ++i) p[i] = r[i] + beta * p[i];
    return rsnew;
}

/* tomography/tv_hpc.F90:162-363 -- split-Bregman TV with an inner CG solve,
 * one slice.  Outputs the FBP warm start (fbp) and the TV result (tv).
 * err_log (optional, nouter entries) receives the print-only Err_diff.   */
static void SFX(tvopt_one)(int N, int T, const float *theta, int wpu,
                           const REAL *f, int ninner, int nouter, int ncg,
                           REAL lambda, REAL mu, int red_mode,
                           REAL *tv, REAL *fbp, double *err_log)
{
    size_t NN = (size_t)N * N, NT = (size_t)N * T;
    REAL *uk = (REAL *)calloc(NN, sizeof(REAL)), *ukp = (REAL *)calloc(NN, sizeof(REAL));
    REAL *dx = (REAL *)calloc(NN, sizeof(REAL)), *dy = (REAL *)calloc(NN, sizeof(REAL));
    REAL *bx = (REAL *)calloc(NN, sizeof(REAL)), *by = (REAL *)calloc(NN, sizeof(REAL));
    REAL *ifkt = (REAL *)calloc(NN, sizeof(REAL)), *rhs = (REAL *)calloc(NN, sizeof(REAL));
    REAL *iukt = (REAL *)calloc(NN, sizeof(REAL)), *r = (REAL *)calloc(NN, sizeof(REAL));
    REAL *p = (REAL *)calloc(NN, sizeof(REAL)), *irpt = (REAL *)calloc(NN, sizeof(REAL));
    REAL *Ap = (REAL *)calloc(NN, sizeof(REAL));
    REAL *fk = (REAL *)calloc(NT, sizeof(REAL)), *ruk = (REAL *)calloc(NT, sizeof(REAL));
    REAL *rp = (REAL *)calloc(NT, sizeof(REAL));
#define AT(a, x, y) (a)[(size_t)((y) - 1) * N + ((x) - 1)]

    SFX(orc_iradon)(N, T, theta, wpu, 1, f, uk);
    if (fbp) memcpy(fbp, uk, NN * sizeof(REAL));
    memcpy(fk, f, NT * sizeof(REAL));

    for (int jouter = 1; jouter <= nouter; ++jouter) {
        double err = 0.0;
        for (int jinner = 1; jinner <= ninner; ++jinner) {
            memcpy(ukp, uk, NN * sizeof(REAL));
            SFX(orc_iradon)(N, T, theta, wpu, 1, fk, ifkt);
            for (int jy = 1; jy <= N; ++jy)
                for (int jx = 1; jx <= N; ++jx) {
                    int jxl = SFX(nb_next)(jx, N), jyl = SFX(nb_next)(jy, N);
                    /* left-to-right, as the Fortran expression */
                    REAL acc = AT(dx, jxl, jy) - AT(bx, jxl, jy);
                    acc = acc - AT(dx, jx, jy);
                    acc = acc + AT(bx, jx, jy);
                    acc = acc + AT(dy, jx, jyl);
                    acc = acc - AT(by, jx, jyl);
                    acc = acc - AT(dy, jx, jy);
                    acc = acc + AT(by, jx, jy);
                    AT(rhs, jx, jy) = mu * AT(ifkt, jx, jy) + lambda * acc;
                }
            SFX(orc_radon)(N, T, theta, 1, uk, ruk);
            SFX(orc_iradon)(N, T, theta, wpu, 1, ruk, iukt);
            for (int jy = 1; jy <= N; ++jy)
                for (int jx = 1; jx <= N; ++jx) {
                    int jxr = SFX(nb_next)(jx, N), jyr = SFX(nb_next)(jy, N);
                    int jxl = SFX(nb_prev)(jx, N), jyl = SFX(nb_prev)(jy, N);
                    REAL lap = (((R(4.0) * AT(uk, jx, jy) - AT(uk, jxl, jy)) - AT(uk, jxr, jy)) - AT(uk, jx, jyl)) - AT(uk, jx, jyr);
                    AT(r, jx, jy) = (AT(rhs, jx, jy) - mu * AT(iukt, jx, jy)) - lambda * lap;
                    AT(p, jx, jy) = AT(r, jx, jy);
                }
            double rsold = SFX(sum_sq)(N, r, red_mode);
            for (int jncg = 1; jncg <= ncg; ++jncg)
                rsold = SFX(orc_cg_step)(N, T, theta, wpu, lambda, mu, red_mode, uk, r, p, Ap, rp, irpt, rsold);
            const REAL thr = R(1.0) / lambda;
            for (int jy = 1; jy <= N; ++jy)
                for (int jx = 1; jx <= N; ++jx) {
                    int jxl = SFX(nb_prev)(jx, N);
                    REAL tmpv = (AT(uk, jxl, jy) - AT(uk, jx, jy)) + AT(bx, jx, jy);
                    REAL dv;
                    if (tmpv == R(0.0)) dv = R(0.0);
                    else dv = (RMAX(RABS(tmpv) - thr, R(0.0)) * tmpv) / RABS(tmpv);
                    AT(dx, jx, jy) = dv;
                    AT(bx, jx, jy) = tmpv - dv;
                    int jyl = SFX(nb_prev)(jy, N);
                    tmpv = (AT(by, jx, jy) + AT(uk, jx, jyl)) - AT(uk, jx, jy);
                    if (tmpv == R(0.0)) dv = R(0.0);
                    else dv = (RMAX(RABS(tmpv) - thr, R(0.0)) * tmpv) / RABS(tmpv);
                    AT(dy, jx, jy) = dv;
                    AT(by, jx, jy) = tmpv - dv;
                }
            err = 0.0;
            for (size_t i = 0; i < NN; ++i) err += RABS(uk[i] - ukp[i]);
        }
        SFX(orc_radon)(N, T, theta, 1, uk, ruk);
        for (size_t i = 0; i < NT; ++i) fk[i] = (fk[i] + f[i]) - ruk[i];
        if (err_log) err_log[jouter - 1] = err;
    }
    memcpy(tv, uk, NN * sizeof(REAL));
#undef AT
    free(uk); free(ukp); free(dx); free(dy); free(bx); free(by); free(ifkt); free(rhs);
    free(iukt); free(r); free(p); free(irpt); free(Ap); free(fk); free(ruk); free(rp);
}

void SFX(orc_tvopt)(int N, int T, const float *theta, int wpu, int S, const REAL *f,
                    int ninner, int nouter, int ncg, REAL lambda, REAL mu, int red_mode,
                    REAL *tv, REAL *fbp)
{
    size_t NN = (size_t)N * N, NT = (size_t)N * T;
    if (S == 1) {
        SFX(tvopt_one)(N, T, theta, wpu, f, ninner, nouter, ncg, lambda, mu, red_mode,
                       tv, fbp, NULL);
        return;
    }
#pragma omp parallel for schedule(dynamic)
    for (int s = 0; s < S; ++s)
        SFX(tvopt_one)(N, T, theta, wpu, f + s * NT, ninner, nouter, ncg, lambda, mu,
                       red_mode, tv + s * NN, fbp ? fbp + s * NN : NULL, NULL);
}
