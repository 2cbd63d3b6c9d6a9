/*
 * flue_oracle.c -- CPU restatement of FLUE's gluonic-observable path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this file; it is used by the test-suite, by the `smoke()` self-check and by
 * the CPU-baseline leg of the benchmark, always as the checker.
 *
 * Parity status: the reference (Fortran 2018, fpm) cannot be compiled on any
 * machine this project builds on (no Fortran compiler) and its own tests hold
 * no golden vectors, so these routines are pinned to analytic known answers
 * (cold fields, abelian constant-flux fields with closed forms, gauge and
 * translation invariance, centre symmetry) and to an independent numpy
 * restatement -- parity against the reference's own binary outputs is
 * unpinned.
 *
 * Every routine follows the reference line by line (file:line cited at each
 * function): same loop nesting, same accumulation order, same association of
 * complex products, FP64 throughout, no fast-math.  Complex numbers are kept
 * as explicit (re, im) pairs and multiplied with the textbook formula, which
 * is what the Fortran compilers emit for `complex(8) * complex(8)`.
 *
 * Memory layout of a gauge field, exactly the reference's
 * `complex(WC) data(NT,NX,NY,NZ,4,3,3)` in Fortran column-major order
 * (src/wloops.F90:60): the 0-based element (t,x,y,z,mu,a,b) lives at complex
 * offset t + NT*(x + NX*(y + NY*(z + NZ*(mu + 4*(a + 3*b))))), with
 * data(..,a,b) = U_ab (row a, column b) and mu = 0,1,2,3 <-> t,x,y,z.  All
 * integer directions, coordinates and path entries at this interface are
 * 1-based, like the reference's.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double re, im;
} cx;
typedef struct {
    cx m[3][3]; /* m[a][b] = U_ab, 0-based */
} mat3;

static inline cx cmul(cx a, cx b) {
    cx r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}
static inline cx cadd(cx a, cx b) {
    cx r = {a.re + b.re, a.im + b.im};
    return r;
}
static inline cx csub(cx a, cx b) {
    cx r = {a.re - b.re, a.im - b.im};
    return r;
}
static inline cx cconj(cx a) {
    cx r = {a.re, -a.im};
    return r;
}
static inline cx cscale(cx a, double s) {
    cx r = {a.re * s, a.im * s};
    return r;
}

typedef struct {
    const double *d; /* interleaved complex128 */
    int64_t n[4];    /* NT, NX, NY, NZ */
    int64_t V;
} field;

static inline int64_t site_of(const field *f, const int c[4]) {
    /* c is 1-based (t,x,y,z) */
    return (int64_t)(c[0] - 1) + f->n[0] * ((int64_t)(c[1] - 1) + f->n[1] * ((int64_t)(c[2] - 1) + f->n[2] * (int64_t)(c[3] - 1)));
}

/* data(c(1),c(2),c(3),c(4),mu,:,:) with mu 1-based */
static inline mat3 link_at(const field *f, const int c[4], int mu) {
    mat3 u;
    int64_t s = site_of(f, c);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            int64_t off = s + f->V * ((int64_t)(mu - 1) + 4 * ((int64_t)a + 3 * (int64_t)b));
            u.m[a][b].re = f->d[2 * off];
            u.m[a][b].im = f->d[2 * off + 1];
        }
    return u;
}

static mat3 ident3(void) {
    /* Ident, src/SU3MatrixOps.f90:7-11 */
    mat3 r;
    memset(&r, 0, sizeof(r));
    r.m[0][0].re = r.m[1][1].re = r.m[2][2].re = 1.0;
    return r;
}

/* MultiplyMatMat, src/SU3MatrixOps.f90:19-37: MM(i,j) = sum_k L(i,k) R(k,j),
 * summed left to right k = 1,2,3. */
static mat3 mulmm(const mat3 *l, const mat3 *r) {
    mat3 o;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            o.m[i][j] = cadd(cadd(cmul(l->m[i][0], r->m[0][j]), cmul(l->m[i][1], r->m[1][j])), cmul(l->m[i][2], r->m[2][j]));
    return o;
}

/* MultiplyMatdagMatdag, src/SU3MatrixOps.f90:39-58:
 * MM(i,j) = conj(sum_k L(k,i) R(j,k)), i.e. MM = L^dagger R^dagger (the
 * reference's comment says (L R)^dagger; the code is followed). */
static mat3 muldd(const mat3 *l, const mat3 *r) {
    mat3 o;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            o.m[i][j] = cconj(cadd(cadd(cmul(l->m[0][i], r->m[j][0]), cmul(l->m[1][i], r->m[j][1])), cmul(l->m[2][i], r->m[j][2])));
    return o;
}

/* TraceMultMatMat, src/SU3MatrixOps.f90:70-80 (exact term order). */
static cx tracemm(const mat3 *l, const mat3 *r) {
    cx t = cmul(l->m[0][0], r->m[0][0]);
    t = cadd(t, cmul(l->m[0][1], r->m[1][0]));
    t = cadd(t, cmul(l->m[0][2], r->m[2][0]));
    t = cadd(t, cmul(l->m[1][0], r->m[0][1]));
    t = cadd(t, cmul(l->m[1][1], r->m[1][1]));
    t = cadd(t, cmul(l->m[1][2], r->m[2][1]));
    t = cadd(t, cmul(l->m[2][0], r->m[0][2]));
    t = cadd(t, cmul(l->m[2][1], r->m[1][2]));
    t = cadd(t, cmul(l->m[2][2], r->m[2][2]));
    return t;
}

/* RealTraceMultMatMat, src/SU3MatrixOps.f90:82-92 */
static double rtracemm(const mat3 *l, const mat3 *r) { return tracemm(l, r).re; }

static mat3 transpose3(const mat3 *a) {
    mat3 o;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) o.m[i][j] = a->m[j][i];
    return o;
}
static mat3 dagger3(const mat3 *a) {
    mat3 o;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) o.m[i][j] = cconj(a->m[j][i]);
    return o;
}

/* periodCoord, src/wloops.F90:546-565: only handles +-1 steps. */
static void period_coord(int c[4], const int64_t n[4]) {
    for (int cc = 0; cc < 4; ++cc) {
        if (c[cc] > n[cc])
            c[cc] = 1;
        else if (c[cc] == 0)
            c[cc] = (int)n[cc];
    }
}

/* genericPath, src/wloops.F90:20-57.  Backward step: move first, then take
 * the dagger of the forward link there (:41-47); forward step: take the link,
 * then move (:48-51); multiply from the right (:54); return the TRANSPOSE of
 * the product (:56). */
static mat3 generic_path(const field *f, const int base[4], const int *path, int npath) {
    int c[4] = {base[0], base[1], base[2], base[3]};
    mat3 u = ident3();
    for (int pp = 0; pp < npath; ++pp) {
        mat3 b = u, a;
        int mu = path[pp];
        int amu = mu < 0 ? -mu : mu;
        if (mu < 0) {
            c[amu - 1] -= 1;
            period_coord(c, f->n);
            mat3 t = link_at(f, c, amu);
            a = dagger3(&t);
        } else {
            a = link_at(f, c, mu);
            c[mu - 1] += 1;
            period_coord(c, f->n);
        }
        u = mulmm(&b, &a);
    }
    return transpose3(&u);
}

static void init_field(field *f, const double *data, int nt, int nx, int ny, int nz) {
    f->d = data;
    f->n[0] = nt;
    f->n[1] = nx;
    f->n[2] = ny;
    f->n[3] = nz;
    f->V = (int64_t)nt * nx * ny * nz;
}

static void store3(double *out, int64_t V, int64_t s, const mat3 *m) {
    /* (NT,NX,NY,NZ,3,3) Fortran order: (s,a,b) at s + V*(a + 3b) */
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            int64_t off = s + V * ((int64_t)a + 3 * (int64_t)b);
            out[2 * off] = m->m[a][b].re;
            out[2 * off + 1] = m->m[a][b].im;
        }
}

static void load_mat(mat3 *m, const double *in) {
    /* one 3x3 complex matrix in Fortran order: (a,b) at a + 3b */
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            m->m[a][b].re = in[2 * (a + 3 * b)];
            m->m[a][b].im = in[2 * (a + 3 * b) + 1];
        }
}
static void save_mat(double *out, const mat3 *m) {
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            out[2 * (a + 3 * b)] = m->m[a][b].re;
            out[2 * (a + 3 * b) + 1] = m->m[a][b].im;
        }
}

/* ------------------------------------------------------------------------ */
/* Exported entry points (ctypes).                                          */
/* ------------------------------------------------------------------------ */

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* MultiplyMatMat / MultiplyMatdagMatdag on single 3x3 Fortran-ordered
 * matrices (c_wrapper/FLUE_c.f90:31-36). */
void oracle_multiplymatmat(double *mm, const double *left, const double *right) {
    mat3 l, r, o;
    load_mat(&l, left);
    load_mat(&r, right);
    o = mulmm(&l, &r);
    save_mat(mm, &o);
}
void oracle_multiplymatdagmatdag(double *mm, const double *left, const double *right) {
    mat3 l, r, o;
    load_mat(&l, left);
    load_mat(&r, right);
    o = muldd(&l, &r);
    save_mat(mm, &o);
}

/* genericPath at one site (src/wloops.F90:20-57). */
void oracle_genericpath(const double *data, int nt, int nx, int ny, int nz, const int *coord_base, const int *path, int npath,
                        double *out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    mat3 u = generic_path(&f, coord_base, path, npath);
    save_mat(out, &u);
}

/* genericPath at every site, output (NT,NX,NY,NZ,3,3). */
void oracle_genericpath_all(const double *data, int nt, int nx, int ny, int nz, const int *path, int npath, double *out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
#pragma omp parallel for collapse(4) schedule(static)
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int t = 1; t <= nt; ++t) {
                    int c[4] = {t, x, y, z};
                    mat3 u = generic_path(&f, c, path, npath);
                    store3(out, f.V, site_of(&f, c), &u);
                }
}

/* genPlaquette, src/wloops.F90:59-127: sum over planes mu in [muStart,muEnd],
 * nu in (mu,nuEnd] and all sites of Re Tr(Ident * genericPath(mu,nu,-mu,-nu)).
 * `parallel` selects the OpenMP collapse(4) reduction of :89 (the
 * reduction order then depends on the thread count). */
void oracle_genplaquette(const double *data, int nt, int nx, int ny, int nz, int mu_start, int mu_end, int nu_end,
                         int parallel, double *sum_out, int64_t *np_out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    mat3 id = ident3();
    double sum = 0.0;
    int64_t np = 0;
    for (int mu = mu_start; mu <= mu_end; ++mu)
        for (int nu = mu + 1; nu <= nu_end; ++nu) {
            int path[4] = {mu, nu, -mu, -nu};
            if (parallel) {
#pragma omp parallel for collapse(4) reduction(+ : sum, np) schedule(static)
                for (int x = 1; x <= nx; ++x)
                    for (int y = 1; y <= ny; ++y)
                        for (int z = 1; z <= nz; ++z)
                            for (int t = 1; t <= nt; ++t) {
                                int c[4] = {t, x, y, z};
                                mat3 p = generic_path(&f, c, path, 4);
                                sum += rtracemm(&id, &p);
                                np += 1;
                            }
            } else {
                for (int x = 1; x <= nx; ++x)
                    for (int y = 1; y <= ny; ++y)
                        for (int z = 1; z <= nz; ++z)
                            for (int t = 1; t <= nt; ++t) {
                                int c[4] = {t, x, y, z};
                                mat3 p = generic_path(&f, c, path, 4);
                                sum += rtracemm(&id, &p);
                                np += 1;
                            }
            }
        }
    *sum_out = sum;
    *np_out = np;
}

/* plaquette, src/wloops.F90:915-1017 (serial, hard-coded links):
 * Re Tr[(U_mu(x) U_nu(x+mu)) (U_mu(x+nu) U_nu(x))^dagger]. */
void oracle_plaquette(const double *data, int nt, int nx, int ny, int nz, int mu_start, int mu_end, int nu_end,
                      double *sum_out, int64_t *np_out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    double sum = 0.0;
    int64_t np = 0;
    for (int mu = mu_start; mu <= mu_end; ++mu) {
        for (int nu = mu + 1; nu <= nu_end; ++nu) {
            for (int x = 1; x <= nx; ++x)
                for (int y = 1; y <= ny; ++y)
                    for (int z = 1; z <= nz; ++z)
                        for (int t = 1; t <= nt; ++t) {
                            int base[4] = {t, x, y, z};
                            int c[4];
                            mat3 umu_x = link_at(&f, base, mu);
                            memcpy(c, base, sizeof(c));
                            c[mu - 1] += 1;
                            for (int cc = 0; cc < 4; ++cc)
                                if (c[cc] > f.n[cc]) c[cc] = 1;
                            mat3 unu_xmu = link_at(&f, c, nu);
                            memcpy(c, base, sizeof(c));
                            c[nu - 1] += 1;
                            for (int cc = 0; cc < 4; ++cc)
                                if (c[cc] > f.n[cc]) c[cc] = 1;
                            mat3 umu_xnu = link_at(&f, c, mu);
                            mat3 unu_x = link_at(&f, base, nu);
                            mat3 a = mulmm(&umu_x, &unu_xmu);
                            mat3 b = muldd(&umu_xnu, &unu_x);
                            sum += rtracemm(&a, &b);
                            np += 1;
                        }
        }
    }
    *sum_out = sum;
    *np_out = np;
}

/* polyakov, src/wloops.F90:1019-1069: for every spatial site the ordered
 * product of U_1(t) over t = 1..NT, then Re Tr.  The reference builds the
 * product as (U(1) U(2) ... U(NT-1)) * U(NT) and only defines it for
 * NT >= 3 (Unu_Temp is set only inside the t loop, :1049-1055); this routine
 * returns -1 for NT < 3. */
int oracle_polyakov(const double *data, int nt, int nx, int ny, int nz, double *sum_out, int64_t *np_out) {
    if (nt < 3) return -1;
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    double sum = 0.0;
    int64_t np = 0;
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z) {
                int c[4] = {1, x, y, z};
                mat3 unu_x = link_at(&f, c, 1), tmp = unu_x;
                for (int t = 2; t <= nt - 1; ++t) {
                    c[0] = t;
                    mat3 unu_xt = link_at(&f, c, 1);
                    tmp = mulmm(&unu_x, &unu_xt);
                    unu_x = tmp;
                }
                c[0] = nt;
                unu_x = link_at(&f, c, 1);
                sum += rtracemm(&tmp, &unu_x);
                np += 1;
            }
    *sum_out = sum;
    *np_out = np;
    return 0;
}

/* Shared body of wmunu (src/wloops.F90:679-791) and wmunutau (:567-677) at
 * one base site: Re Tr[(U^nMu_mu(x) U^nNu_nu(x+nMu mu)) (U^nMu_mu(x+nNu nu) U^nNu_nu(x))^dagger]. */
static double wloop_site(const field *f, const int base[4], int mu, int nu, int nmu, int nnu) {
    int muc[4] = {0, 0, 0, 0}, nuc[4] = {0, 0, 0, 0}, c[4];
    muc[mu - 1] = 1;
    nuc[nu - 1] = 1;
    mat3 umu_x, unu_xpamuh, umu_xpanuh, unu_x, utemp, utemp2;
#define STEP(v)                                               \
    do {                                                      \
        for (int k = 0; k < 4; ++k) c[k] += v[k];             \
        period_coord(c, f->n);                                \
    } while (0)
    /* U_nMu(x) */
    memcpy(c, base, sizeof(c));
    umu_x = ident3();
    for (int nn = 1; nn <= nmu; ++nn) {
        utemp = link_at(f, c, mu);
        utemp2 = mulmm(&umu_x, &utemp);
        umu_x = utemp2;
        STEP(muc);
    }
    /* U_nNu(x + nMu mu) */
    memcpy(c, base, sizeof(c));
    STEP(muc);
    for (int nn = 2; nn <= nmu; ++nn) STEP(muc);
    unu_xpamuh = ident3();
    for (int nn = 1; nn <= nnu; ++nn) {
        utemp = link_at(f, c, nu);
        utemp2 = mulmm(&unu_xpamuh, &utemp);
        unu_xpamuh = utemp2;
        STEP(nuc);
    }
    /* U_nMu(x + nNu nu) */
    memcpy(c, base, sizeof(c));
    STEP(nuc);
    for (int nn = 2; nn <= nnu; ++nn) STEP(nuc);
    umu_xpanuh = ident3();
    for (int nn = 1; nn <= nmu; ++nn) {
        utemp = link_at(f, c, mu);
        utemp2 = mulmm(&umu_xpanuh, &utemp);
        umu_xpanuh = utemp2;
        STEP(muc);
    }
    /* U_nNu(x) */
    memcpy(c, base, sizeof(c));
    unu_x = ident3();
    for (int nn = 1; nn <= nnu; ++nn) {
        utemp = link_at(f, c, nu);
        utemp2 = mulmm(&unu_x, &utemp);
        unu_x = utemp2;
        STEP(nuc);
    }
#undef STEP
    mat3 a = mulmm(&umu_x, &unu_xpamuh);
    mat3 b = muldd(&umu_xpanuh, &unu_x);
    return rtracemm(&a, &b);
}

/* parallel != 0: the same per-site loops under an OpenMP reduction (only the
 * order of the FP64 sum over sites differs), for full-size lattices. */
double oracle_wmunu(const double *data, int nt, int nx, int ny, int nz, int mu, int nu, int nmu, int nnu,
                    int parallel) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    double v = 0.0;
    if (parallel) {
#pragma omp parallel for collapse(4) reduction(+ : v) schedule(static)
        for (int x = 1; x <= nx; ++x)
            for (int y = 1; y <= ny; ++y)
                for (int z = 1; z <= nz; ++z)
                    for (int t = 1; t <= nt; ++t) {
                        int base[4] = {t, x, y, z};
                        v += wloop_site(&f, base, mu, nu, nmu, nnu);
                    }
        return v / (double)f.V;
    }
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int t = 1; t <= nt; ++t) {
                    int base[4] = {t, x, y, z};
                    v += wloop_site(&f, base, mu, nu, nmu, nnu);
                }
    return v / (double)f.V;
}

double oracle_wmunutau(const double *data, int nt, int nx, int ny, int nz, int tau, int mu, int nu, int nmu, int nnu) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    double v = 0.0;
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z) {
                int base[4] = {tau, x, y, z};
                v += wloop_site(&f, base, mu, nu, nmu, nnu);
            }
    return v / (double)(nx * ny * nz);
}

/* Projection used by cloverLoopMuNuCoord (src/wloops.F90:178-190) and
 * Loop5MuNuCoord (:411-423): anti-Hermitian, NOT traceless, times 1/4. */
static mat3 ah_quarter(mat3 u) {
    cx c12 = cscale(csub(u.m[0][1], cconj(u.m[1][0])), 0.5);
    cx c13 = cscale(csub(u.m[0][2], cconj(u.m[2][0])), 0.5);
    cx c23 = cscale(csub(u.m[1][2], cconj(u.m[2][1])), 0.5);
    u.m[0][1] = c12;
    u.m[0][2] = c13;
    u.m[1][2] = c23;
    u.m[1][0] = cscale(cconj(c12), -1.0);
    u.m[2][0] = cscale(cconj(c13), -1.0);
    u.m[2][1] = cscale(cconj(c23), -1.0);
    for (int i = 0; i < 3; ++i) {
        u.m[i][i].re = 0.0;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) u.m[i][j] = cscale(u.m[i][j], 0.25);
    return u;
}

static void madd(mat3 *acc, const mat3 *b) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) acc->m[i][j] = cadd(acc->m[i][j], b->m[i][j]);
}
static mat3 mscale(mat3 a, double s) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a.m[i][j] = cscale(a.m[i][j], s);
    return a;
}

/* cloverLoopMuNuCoord, src/wloops.F90:129-199 */
static mat3 clover_site(const field *f, const int base[4], int mu, int nu) {
    int p[4][4] = {{nu, -mu, -nu, mu}, {mu, nu, -mu, -nu}, {-mu, -nu, mu, nu}, {-nu, mu, nu, -mu}};
    mat3 u = generic_path(f, base, p[0], 4);
    for (int k = 1; k < 4; ++k) {
        mat3 l = generic_path(f, base, p[k], 4);
        madd(&u, &l);
    }
    return ah_quarter(u);
}

void oracle_clover(const double *data, int nt, int nx, int ny, int nz, int mu, int nu, double *out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
#pragma omp parallel for collapse(4) schedule(static)
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int t = 1; t <= nt; ++t) {
                    int c[4] = {t, x, y, z};
                    mat3 u = clover_site(&f, c, mu, nu);
                    store3(out, f.V, site_of(&f, c), &u);
                }
}

/* Loop5MuNuCoord, src/wloops.F90:201-432 (hep-lat/0203008).  Coefficients
 * :219-224, path tables :236-290, accumulation order :313-405, projection
 * :411-423. */
static void loop5_paths(int mu, int nu, int p11[4][4], int p22[4][8], int p33[4][12], int p12[8][6], int p13[8][8]) {
    int a11[4][4] = {{nu, -mu, -nu, mu}, {mu, nu, -mu, -nu}, {-mu, -nu, mu, nu}, {-nu, mu, nu, -mu}};
    int a22[4][8] = {{nu, nu, -mu, -mu, -nu, -nu, mu, mu},
                     {mu, mu, nu, nu, -mu, -mu, -nu, -nu},
                     {-mu, -mu, -nu, -nu, mu, mu, nu, nu},
                     {-nu, -nu, mu, mu, nu, nu, -mu, -mu}};
    int a33[4][12] = {{nu, nu, nu, -mu, -mu, -mu, -nu, -nu, -nu, mu, mu, mu},
                      {mu, mu, mu, nu, nu, nu, -mu, -mu, -mu, -nu, -nu, -nu},
                      {-mu, -mu, -mu, -nu, -nu, -nu, mu, mu, mu, nu, nu, nu},
                      {-nu, -nu, -nu, mu, mu, mu, nu, nu, nu, -mu, -mu, -mu}};
    int a12[8][6] = {{nu, nu, -mu, -nu, -nu, mu},   {mu, nu, nu, -mu, -nu, -nu},   {-mu, -nu, -nu, mu, nu, nu},
                     {-nu, -nu, mu, nu, nu, -mu},   {nu, -mu, -mu, -nu, mu, mu},   {mu, mu, nu, -mu, -mu, -nu},
                     {-mu, -mu, -nu, mu, mu, nu},   {-nu, mu, mu, nu, -mu, -mu}};
    int a13[8][8] = {{nu, nu, nu, -mu, -nu, -nu, -nu, mu}, {mu, nu, nu, nu, -mu, -nu, -nu, -nu},
                     {-mu, -nu, -nu, -nu, mu, nu, nu, nu}, {-nu, -nu, -nu, mu, nu, nu, nu, -mu},
                     {nu, -mu, -mu, -mu, -nu, mu, mu, mu}, {mu, mu, mu, nu, -mu, -mu, -mu, -nu},
                     {-mu, -mu, -mu, -nu, mu, mu, mu, nu}, {-nu, mu, mu, mu, nu, -mu, -mu, -mu}};
    memcpy(p11, a11, sizeof(a11));
    memcpy(p22, a22, sizeof(a22));
    memcpy(p33, a33, sizeof(a33));
    memcpy(p12, a12, sizeof(a12));
    memcpy(p13, a13, sizeof(a13));
}

static const double K5 = 1.0 / 180.0;
#define K1 ((19.0 / 9.0) - 55.0 * K5)
#define K2 ((1.0 / 36.0) - 16.0 * K5)
#define K3 (64.0 * K5 - (32.0 / 45.0))
#define K4 ((1.0 / 15.0) - 6.0 * K5)

/* Q before projection (the sum of :313-405), and the projected F. */
static mat3 loop5_sum_site(const field *f, const int base[4], int mu, int nu) {
    int p11[4][4], p22[4][8], p33[4][12], p12[8][6], p13[8][8];
    loop5_paths(mu, nu, p11, p22, p33, p12, p13);
    mat3 thisu, worku, l;
    /* 1x1 */
    thisu = generic_path(f, base, p11[0], 4);
    for (int k = 1; k < 4; ++k) {
        l = generic_path(f, base, p11[k], 4);
        madd(&thisu, &l);
    }
    thisu = mscale(thisu, K1);
    /* 2x2 */
    worku = generic_path(f, base, p22[0], 8);
    for (int k = 1; k < 4; ++k) {
        l = generic_path(f, base, p22[k], 8);
        madd(&worku, &l);
    }
    worku = mscale(worku, K2);
    madd(&thisu, &worku);
    /* 3x3 */
    worku = generic_path(f, base, p33[0], 12);
    for (int k = 1; k < 4; ++k) {
        l = generic_path(f, base, p33[k], 12);
        madd(&worku, &l);
    }
    worku = mscale(worku, K5);
    madd(&thisu, &worku);
    /* 1x2: order 1,5,2,6,3,7,4,8 (:362-381) */
    static const int ord[8] = {0, 4, 1, 5, 2, 6, 3, 7};
    worku = generic_path(f, base, p12[ord[0]], 6);
    for (int k = 1; k < 8; ++k) {
        l = generic_path(f, base, p12[ord[k]], 6);
        madd(&worku, &l);
    }
    worku = mscale(mscale(worku, K3), 0.5);
    madd(&thisu, &worku);
    /* 1x3 (:386-405) */
    worku = generic_path(f, base, p13[ord[0]], 8);
    for (int k = 1; k < 8; ++k) {
        l = generic_path(f, base, p13[ord[k]], 8);
        madd(&worku, &l);
    }
    worku = mscale(mscale(worku, K4), 0.5);
    madd(&thisu, &worku);
    return thisu;
}

void oracle_loop5(const double *data, int nt, int nx, int ny, int nz, int mu, int nu, double *out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
#pragma omp parallel for collapse(4) schedule(static)
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int t = 1; t <= nt; ++t) {
                    int c[4] = {t, x, y, z};
                    mat3 u = ah_quarter(loop5_sum_site(&f, c, mu, nu));
                    store3(out, f.V, site_of(&f, c), &u);
                }
}

/* magnetic, src/wloops.F90:479-544: B^2 = (1/V) sum_x sum_i -Re Tr(F_i F_i)
 * with F_1 = Loop5(3,2), F_2 = Loop5(2,4), F_3 = Loop5(4,3) (:502-506).
 * Instead of the 3-plane full-volume BField temporary the per-site F are
 * formed and consumed in the same (x,y,z,t,ii) order as the reduction loop
 * :517-533, which gives the same serial sum.  `parallel` selects the OpenMP
 * collapse(5) reduction of :514. */
double oracle_magnetic(const double *data, int nt, int nx, int ny, int nz, int parallel) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    static const int planes[3][2] = {{3, 2}, {2, 4}, {4, 3}};
    double cp = 0.0;
    if (parallel) {
#pragma omp parallel for collapse(4) reduction(+ : cp) schedule(static)
        for (int x = 1; x <= nx; ++x)
            for (int y = 1; y <= ny; ++y)
                for (int z = 1; z <= nz; ++z)
                    for (int t = 1; t <= nt; ++t) {
                        int c[4] = {t, x, y, z};
                        for (int ii = 0; ii < 3; ++ii) {
                            mat3 fm = ah_quarter(loop5_sum_site(&f, c, planes[ii][0], planes[ii][1]));
                            cp = cp - rtracemm(&fm, &fm);
                        }
                    }
    } else {
        for (int x = 1; x <= nx; ++x)
            for (int y = 1; y <= ny; ++y)
                for (int z = 1; z <= nz; ++z)
                    for (int t = 1; t <= nt; ++t) {
                        int c[4] = {t, x, y, z};
                        for (int ii = 0; ii < 3; ++ii) {
                            mat3 fm = ah_quarter(loop5_sum_site(&f, c, planes[ii][0], planes[ii][1]));
                            cp = cp - rtracemm(&fm, &fm);
                        }
                    }
    }
    return cp / (double)f.V;
}

/* The magnetic() sum restricted to the time slices t in [t_begin, t_end]
 * (1-based) of a full field, OpenMP over sites: the bounded CPU sample used by
 * the benchmark's CPU-baseline leg.  Returns the raw sum of -Re Tr(F F). */
double oracle_magnetic_slab(const double *data, int nt, int nx, int ny, int nz, int t_begin, int t_end) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    static const int planes[3][2] = {{3, 2}, {2, 4}, {4, 3}};
    double cp = 0.0;
#pragma omp parallel for collapse(4) reduction(+ : cp) schedule(static)
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int t = t_begin; t <= t_end; ++t) {
                    int c[4] = {t, x, y, z};
                    for (int ii = 0; ii < 3; ++ii) {
                        mat3 fm = ah_quarter(loop5_sum_site(&f, c, planes[ii][0], planes[ii][1]));
                        cp = cp - rtracemm(&fm, &fm);
                    }
                }
    return cp;
}

/* B^2-style energy over an arbitrary set of 5-loop planes (used to check the
 * generalised energy and its gradient): sum over listed (mu,nu) pairs of
 * -Re Tr(F F), divided by V. */
double oracle_loop5_energy(const double *data, int nt, int nx, int ny, int nz, const int *planes, int nplanes) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    double cp = 0.0;
#pragma omp parallel for collapse(4) reduction(+ : cp) schedule(static)
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int t = 1; t <= nt; ++t) {
                    int c[4] = {t, x, y, z};
                    for (int ii = 0; ii < nplanes; ++ii) {
                        mat3 fm = ah_quarter(loop5_sum_site(&f, c, planes[2 * ii], planes[2 * ii + 1]));
                        cp = cp - rtracemm(&fm, &fm);
                    }
                }
    return cp / (double)f.V;
}

/* ------------------------------------------------------------------------ */
/* FixSU3Matrix and helpers, src/gaugeIO/ILDG_bin.f90:108-159.              */
/* ------------------------------------------------------------------------ */
static void orthogonalise(cx w[3], const cx v[3]) {
    /* :108-118: w = w - v * sum(conjg(v) * w) */
    cx d = cmul(cconj(v[0]), w[0]);
    d = cadd(d, cmul(cconj(v[1]), w[1]));
    d = cadd(d, cmul(cconj(v[2]), w[2]));
    for (int i = 0; i < 3; ++i) w[i] = csub(w[i], cmul(v[i], d));
}
static void vector_product(cx x[3], const cx v[3], const cx w[3]) {
    /* :120-135: x(i) = conjg(v(j) w(k) - v(k) w(j)), (i,j,k) cyclic */
    for (int ic = 0; ic < 3; ++ic) {
        int jc = (ic + 1) % 3, kc = (jc + 1) % 3;
        x[ic] = cconj(csub(cmul(v[jc], w[kc]), cmul(v[kc], w[jc])));
    }
}
static void normalise(cx v[3]) {
    /* :154-159 */
    double n = sqrt((v[0].re * v[0].re + v[0].im * v[0].im) + (v[1].re * v[1].re + v[1].im * v[1].im) +
                    (v[2].re * v[2].re + v[2].im * v[2].im));
    for (int i = 0; i < 3; ++i) {
        v[i].re /= n;
        v[i].im /= n;
    }
}
static void fix_su3(mat3 *u) {
    /* :138-151 */
    cx v1[3], v2[3], v3[3];
    for (int i = 0; i < 3; ++i) v1[i] = u->m[0][i];
    normalise(v1);
    for (int i = 0; i < 3; ++i) v2[i] = u->m[1][i];
    orthogonalise(v2, v1);
    normalise(v2);
    vector_product(v3, v1, v2);
    normalise(v3);
    for (int i = 0; i < 3; ++i) {
        u->m[0][i] = v1[i];
        u->m[1][i] = v2[i];
        u->m[2][i] = v3[i];
    }
}

/* FixSU3Matrix applied to one 3x3 Fortran-ordered matrix in place. */
void oracle_fixsu3matrix(double *u) {
    mat3 m;
    load_mat(&m, u);
    fix_su3(&m);
    save_mat(u, &m);
}

/* FixSU3Matrix applied to every link of a field in place. */
void oracle_fixsu3_field(double *data, int nt, int nx, int ny, int nz) {
    int64_t V = (int64_t)nt * nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int64_t sm = 0; sm < 4 * V; ++sm) {
        mat3 m;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                int64_t off = sm + 4 * V * ((int64_t)a + 3 * b);
                m.m[a][b].re = data[2 * off];
                m.m[a][b].im = data[2 * off + 1];
            }
        fix_su3(&m);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                int64_t off = sm + 4 * V * ((int64_t)a + 3 * b);
                data[2 * off] = m.m[a][b].re;
                data[2 * off + 1] = m.m[a][b].im;
            }
    }
}

/* ------------------------------------------------------------------------ */
/* uzerobar.  No reference code exists (README.md:17 only); definitions:    */
/*   plaquette u0:  u0 = (<Re Tr P>/3)^(1/4) over all / spatial planes,     */
/*                  u_t = (<Re Tr P_st>/3)^(1/2) / u_s                       */
/*   Landau mean link: u0_L = <Re Tr(G(x) U_mu(x) G(x+mu)^dagger)>/3 over   */
/*                  all, spatial (mu=2..4) and temporal (mu=1) links.       */
/* G is (NT,NX,NY,NZ,3,3) Fortran order like ReadGaugeTransformation_cola's */
/* result (src/gaugeIO/ILDG_bin.f90:65-105), or NULL.                       */
/* out: [u0_all, u0_s, u0_t, uL_all, uL_s, uL_t]                            */
/* ------------------------------------------------------------------------ */
void oracle_uzerobar(const double *data, int nt, int nx, int ny, int nz, const double *g, double *out) {
    double s_all, s_s, s_t;
    int64_t n_all, n_s, n_t;
    oracle_plaquette(data, nt, nx, ny, nz, 1, 4, 4, &s_all, &n_all);
    oracle_plaquette(data, nt, nx, ny, nz, 2, 4, 4, &s_s, &n_s);
    oracle_plaquette(data, nt, nx, ny, nz, 1, 1, 4, &s_t, &n_t);
    double p_all = s_all / (double)n_all / 3.0, p_s = s_s / (double)n_s / 3.0, p_t = s_t / (double)n_t / 3.0;
    out[0] = pow(p_all, 0.25);
    out[1] = pow(p_s, 0.25);
    out[2] = sqrt(p_t) / out[1];
    out[3] = out[4] = out[5] = NAN;
    if (!g) return;
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    double lsum[4] = {0, 0, 0, 0};
    for (int mu = 1; mu <= 4; ++mu) {
        double acc = 0.0;
        for (int x = 1; x <= nx; ++x)
            for (int y = 1; y <= ny; ++y)
                for (int z = 1; z <= nz; ++z)
                    for (int t = 1; t <= nt; ++t) {
                        int c[4] = {t, x, y, z}, cp[4] = {t, x, y, z};
                        cp[mu - 1] += 1;
                        period_coord(cp, f.n);
                        mat3 gx, gxp, u = link_at(&f, c, mu);
                        int64_t s = site_of(&f, c), sp = site_of(&f, cp);
                        for (int a = 0; a < 3; ++a)
                            for (int b = 0; b < 3; ++b) {
                                int64_t o1 = s + f.V * (a + 3 * b), o2 = sp + f.V * (a + 3 * b);
                                gx.m[a][b].re = g[2 * o1];
                                gx.m[a][b].im = g[2 * o1 + 1];
                                gxp.m[a][b].re = g[2 * o2];
                                gxp.m[a][b].im = g[2 * o2 + 1];
                            }
                        mat3 gu = mulmm(&gx, &u), gpd = dagger3(&gxp);
                        acc += rtracemm(&gu, &gpd);
                    }
        lsum[mu - 1] = acc;
    }
    double V = (double)f.V;
    out[3] = (lsum[0] + lsum[1] + lsum[2] + lsum[3]) / (4.0 * V) / 3.0;
    out[4] = (lsum[1] + lsum[2] + lsum[3]) / (3.0 * V) / 3.0;
    out[5] = lsum[0] / V / 3.0;
}

/* ------------------------------------------------------------------------ */
/* Gradients (no reference counterpart).  Conventions: for an observable O  */
/* and a link U = U_mu(x), N is the matrix with dO = Re Tr(dU N) for every  */
/* variation dU; the su(3)-projected Lie gradient is                         */
/*   G = sum_a T^a d/dh O(e^{h T^a} U) = -1/2 TA(U N),  T^a = i lambda^a/2,  */
/* TA(M) = (M - M^dagger)/2 - Tr((M - M^dagger)/2)/3.  Output layout is the */
/* field layout (NT,NX,NY,NZ,4,3,3).                                         */
/* ------------------------------------------------------------------------ */
static void store_link(double *out, int64_t V, int64_t s, int mu0, const mat3 *m) {
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            int64_t off = s + V * ((int64_t)mu0 + 4 * ((int64_t)a + 3 * b));
            out[2 * off] = m->m[a][b].re;
            out[2 * off + 1] = m->m[a][b].im;
        }
}
static mat3 lie_project(const mat3 *u, const mat3 *n) {
    mat3 m = mulmm(u, n), g;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            cx a = m.m[i][j], b = cconj(m.m[j][i]);
            g.m[i][j] = cscale(csub(a, b), 0.5);
        }
    double tr = (g.m[0][0].im + g.m[1][1].im + g.m[2][2].im) / 3.0;
    for (int i = 0; i < 3; ++i) g.m[i][i].im -= tr;
    return mscale(g, -0.5);
}

/* Analytic Wilson staple force of O = sum_{x, mu<nu} Re Tr P_munu(x):
 * N_mu(x) = sum_{nu != mu} [U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+
 *                          + U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu)].
 * Writes the Lie gradient G for every link. */
void oracle_plaquette_staple_force(const double *data, int nt, int nx, int ny, int nz, double *out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
#pragma omp parallel for collapse(4) schedule(static)
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int t = 1; t <= nt; ++t) {
                    int c[4] = {t, x, y, z};
                    for (int mu = 1; mu <= 4; ++mu) {
                        mat3 n;
                        memset(&n, 0, sizeof(n));
                        for (int nu = 1; nu <= 4; ++nu) {
                            if (nu == mu) continue;
                            int cm[4], cn[4], cmn[4], cmnn[4];
                            memcpy(cm, c, sizeof(c));
                            cm[mu - 1] += 1;
                            period_coord(cm, f.n);
                            memcpy(cn, c, sizeof(c));
                            cn[nu - 1] += 1;
                            period_coord(cn, f.n);
                            memcpy(cmn, c, sizeof(c));
                            cmn[nu - 1] -= 1;
                            period_coord(cmn, f.n); /* x - nu */
                            memcpy(cmnn, cmn, sizeof(c));
                            cmnn[mu - 1] += 1;
                            period_coord(cmnn, f.n); /* x + mu - nu */
                            mat3 a = link_at(&f, cm, nu), b = link_at(&f, cn, mu), d = link_at(&f, c, nu);
                            mat3 bd = dagger3(&b), dd = dagger3(&d);
                            mat3 t1 = mulmm(&a, &bd);
                            mat3 up = mulmm(&t1, &dd);
                            mat3 e = link_at(&f, cmnn, nu), g2 = link_at(&f, cmn, mu), h = link_at(&f, cmn, nu);
                            mat3 ed = dagger3(&e), gd = dagger3(&g2);
                            mat3 t2 = mulmm(&ed, &gd);
                            mat3 dn = mulmm(&t2, &h);
                            madd(&n, &up);
                            madd(&n, &dn);
                        }
                        mat3 u = link_at(&f, c, mu);
                        mat3 g = lie_project(&u, &n);
                        store_link(out, f.V, site_of(&f, c), mu - 1, &g);
                    }
                }
}

/* Gradient of E = sum over listed planes of sum_x -Re Tr(F F) / V with the
 * 5-loop F, by brute-force reverse mode over every path of every site: for
 * a leaf W = L_1 ... L_n (transposed by genericPath, which the energy does
 * not see) with cotangent K at its base, the link of step k receives
 * L_{k+1} ... L_n K L_1 ... L_{k-1} (forward step) or the dagger-rule
 * equivalent (backward step).  Serial scatter; an independent formulation
 * from the GPU kernels'. Output: Lie gradient G per link. */
static void scatter_path(const field *f, const int base[4], const int *path, int npath, const mat3 *kmat, mat3 *nacc) {
    /* positions and links of the path */
    int c[4] = {base[0], base[1], base[2], base[3]};
    mat3 lk[12];
    int64_t lsite[12];
    int ldir[12], lback[12];
    for (int pp = 0; pp < npath; ++pp) {
        int mu = path[pp], amu = mu < 0 ? -mu : mu;
        if (mu < 0) {
            c[amu - 1] -= 1;
            period_coord(c, f->n);
            mat3 t = link_at(f, c, amu);
            lk[pp] = dagger3(&t);
            lback[pp] = 1;
        } else {
            lk[pp] = link_at(f, c, mu);
            lback[pp] = 0;
        }
        lsite[pp] = site_of(f, c);
        ldir[pp] = amu - 1;
        if (mu > 0) {
            c[mu - 1] += 1;
            period_coord(c, f->n);
        }
    }
    for (int k = 0; k < npath; ++k) {
        /* R = L_{k+1} ... L_n K L_1 ... L_{k-1} */
        mat3 r = ident3();
        for (int j = k + 1; j < npath; ++j) r = mulmm(&r, &lk[j]);
        r = mulmm(&r, kmat);
        for (int j = 0; j < k; ++j) r = mulmm(&r, &lk[j]);
        /* dE = Re Tr(dL_k R).  forward: dL = dU -> N += R.
         * backward: dL = dU^+ -> Re Tr(dU^+ R) = Re Tr(dU R^+) -> N += R^+ */
        mat3 add = lback[k] ? dagger3(&r) : r;
        mat3 *dst = &nacc[lsite[k] * 4 + ldir[k]];
        madd(dst, &add);
    }
}

void oracle_loop5_energy_force(const double *data, int nt, int nx, int ny, int nz, const int *planes, int nplanes,
                               double *out) {
    field f;
    init_field(&f, data, nt, nx, ny, nz);
    int64_t V = f.V;
    mat3 *nacc = (mat3 *)calloc((size_t)V * 4, sizeof(mat3));
    for (int ip = 0; ip < nplanes; ++ip) {
        int mu = planes[2 * ip], nu = planes[2 * ip + 1];
        int p11[4][4], p22[4][8], p33[4][12], p12[8][6], p13[8][8];
        loop5_paths(mu, nu, p11, p22, p33, p12, p13);
        for (int x = 1; x <= nx; ++x)
            for (int y = 1; y <= ny; ++y)
                for (int z = 1; z <= nz; ++z)
                    for (int t = 1; t <= nt; ++t) {
                        int c[4] = {t, x, y, z};
                        mat3 fm = ah_quarter(loop5_sum_site(&f, c, mu, nu));
                        /* The leaves are transposed path products W^T and
                         * F = AH(Q)/4 with Q = sum c W^T; with Ft = F^T the
                         * non-transposed field strength, E = -1/V Re Tr(Ft Ft),
                         * dE = -(1/(2V)) Re Tr(Ft dQt), Qt = sum c W. */
                        mat3 ft = transpose3(&fm);
                        mat3 k = mscale(ft, -1.0 / (2.0 * (double)V));
                        mat3 kc;
                        kc = mscale(k, K1);
                        for (int q = 0; q < 4; ++q) scatter_path(&f, c, p11[q], 4, &kc, nacc);
                        kc = mscale(k, K2);
                        for (int q = 0; q < 4; ++q) scatter_path(&f, c, p22[q], 8, &kc, nacc);
                        kc = mscale(k, K5);
                        for (int q = 0; q < 4; ++q) scatter_path(&f, c, p33[q], 12, &kc, nacc);
                        kc = mscale(k, K3 * 0.5);
                        for (int q = 0; q < 8; ++q) scatter_path(&f, c, p12[q], 6, &kc, nacc);
                        kc = mscale(k, K4 * 0.5);
                        for (int q = 0; q < 8; ++q) scatter_path(&f, c, p13[q], 8, &kc, nacc);
                    }
    }
    for (int64_t s = 0; s < V; ++s) {
        int64_t r = s;
        int c[4];
        c[0] = (int)(r % nt) + 1;
        r /= nt;
        c[1] = (int)(r % nx) + 1;
        r /= nx;
        c[2] = (int)(r % ny) + 1;
        r /= ny;
        c[3] = (int)r + 1;
        for (int mu = 1; mu <= 4; ++mu) {
            mat3 u = link_at(&f, c, mu);
            mat3 g = lie_project(&u, &nacc[s * 4 + mu - 1]);
            store_link(out, V, s, mu - 1, &g);
        }
    }
    free(nacc);
}
