/*
 * simp_oracle.c -- FP64 CPU oracle for the 3D SIMP hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker that the CUDA library is compared
 * against (tests/, __graft_entry__.smoke()) and the timed CPU baseline of bench.py. The
 * product path never links, loads or calls it.
 *
 * It restates, in plain C with OpenMP, the algorithm of the reference CPU solver
 * genpipeline/topology/simp_solver.py (class SIMPSolver):
 *   - element/DOF numbering          simp_solver.py:251-282 (_build_edof_mapping)
 *   - global K(x) = sum_e E(x_e) Ke  simp_solver.py:200-205 (COO assembly in _sensitivity)
 *   - u solve on the free DOFs       simp_solver.py:207-213 (spsolve on K[free][:,free])
 *   - ce, dc                         simp_solver.py:215-218
 *   - density filter H, Hs           simp_solver.py:1545-1567 (_build_filter)
 *   - sensitivity chain rule         simp_solver.py:221-223 (_filter_dc)
 *   - OC bisection                   simp_solver.py:225-249 (_oc_update); the parameters of
 *                                    the GPU variant simp_solver_gpu.py:801-841 are accepted
 *   - the SIMP loop                  simp_solver.py:56-79 (run)
 * The direct sparse solve is replaced by matrix-free Jacobi-PCG in FP64 (the loop of
 * simp_solver_gpu.py:328-379 without its early exits) driven to a tight tolerance; at
 * small sizes the tests check it against the reference's spsolve solutions.
 *
 * Conventions (reference): element e = i*ny*nz + j*nz + k; node n = i*(ny+1)*(nz+1) +
 * j*(nz+1) + k; DOF 3n+c; local node a in the order (0,0,0),(1,0,0),(1,1,0),(0,1,0),
 * (0,0,1),(1,0,1),(1,1,1),(0,1,1).
 *
 * Stiffness laws:  law 0 ("ref")      E = e0 * max(x, xmin)^p,  dE/dx = e0 p max(x,xmin)^(p-1)
 *                  law 1 ("modified") E = emin + x^p (e0-emin),  dE/dx = p x^(p-1) (e0-emin)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static const int ORC_CORNER[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* Unit-cube trilinear hexahedron stiffness, 2x2x2 Gauss quadrature of B^T D B
 * (isotropic, Young's modulus e0, Poisson ratio nu). Engineering shear strains (xy,yz,zx). */
void orc_ke_quadrature(double nu, double e0, double *ke) {
    double lam = e0 * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double mu = e0 / (2.0 * (1.0 + nu));
    double d[6][6];
    memset(d, 0, sizeof d);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) d[i][j] = lam;
    for (int i = 0; i < 3; ++i) {
        d[i][i] = lam + 2.0 * mu;
        d[3 + i][3 + i] = mu;
    }
    double g[2] = {0.5 - 0.5 / sqrt(3.0), 0.5 + 0.5 / sqrt(3.0)};
    memset(ke, 0, 576 * sizeof(double));
    for (int qx = 0; qx < 2; ++qx)
        for (int qy = 0; qy < 2; ++qy)
            for (int qz = 0; qz < 2; ++qz) {
                double b[6][24];
                memset(b, 0, sizeof b);
                for (int a = 0; a < 8; ++a) {
                    int cx = ORC_CORNER[a][0], cy = ORC_CORNER[a][1], cz = ORC_CORNER[a][2];
                    double fx = cx ? g[qx] : 1.0 - g[qx];
                    double fy = cy ? g[qy] : 1.0 - g[qy];
                    double fz = cz ? g[qz] : 1.0 - g[qz];
                    double dx = (cx ? 1.0 : -1.0) * fy * fz;
                    double dy = fx * (cy ? 1.0 : -1.0) * fz;
                    double dz = fx * fy * (cz ? 1.0 : -1.0);
                    b[0][3 * a] = dx;
                    b[1][3 * a + 1] = dy;
                    b[2][3 * a + 2] = dz;
                    b[3][3 * a] = dy;
                    b[3][3 * a + 1] = dx;
                    b[4][3 * a + 1] = dz;
                    b[4][3 * a + 2] = dy;
                    b[5][3 * a] = dz;
                    b[5][3 * a + 2] = dx;
                }
                for (int r = 0; r < 24; ++r)
                    for (int c = 0; c < 24; ++c) {
                        double s = 0.0;
                        for (int m = 0; m < 6; ++m)
                            for (int n = 0; n < 6; ++n) s += b[m][r] * d[m][n] * b[n][c];
                        ke[r * 24 + c] += s / 8.0;
                    }
            }
    for (int r = 0; r < 24; ++r)
        for (int c = r + 1; c < 24; ++c) {
            double s = 0.5 * (ke[r * 24 + c] + ke[c * 24 + r]);
            ke[r * 24 + c] = s;
            ke[c * 24 + r] = s;
        }
}

static inline double orc_E(int law, double x, double penal, double e0, double emin, double xmin) {
    if (law == 0) return e0 * pow(x > xmin ? x : xmin, penal);
    return emin + pow(x, penal) * (e0 - emin);
}

static inline double orc_dE(int law, double x, double penal, double e0, double emin, double xmin) {
    if (law == 0) return e0 * penal * pow(x > xmin ? x : xmin, penal - 1.0);
    return penal * pow(x, penal - 1.0) * (e0 - emin);
}

/* E(x_e) for every element. */
void orc_moduli(int64_t n_elem, const double *x, int law, double penal, double e0, double emin,
                double xmin, double *E) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n_elem; ++e) E[e] = orc_E(law, x[e], penal, e0, emin, xmin);
}

/* y = D K(x) D p, K(x) = sum_e E_e P_e^T Ke P_e (simp_solver.py:200-205); D zeroes the DOFs
 * flagged in fixed (nullable: no masking). Each node gathers from its <= 8 elements, so the
 * sum for one DOF is taken in a fixed order. */
void orc_apply(int nx, int ny, int nz, const double *ke, const double *E, const double *p,
               const uint8_t *fixed, double *y) {
    const int64_t NY = ny + 1, NZ = nz + 1;
    const int64_t n_nodes = (int64_t)(nx + 1) * NY * NZ;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < n_nodes; ++n) {
        int i = (int)(n / (NY * NZ)), j = (int)((n / NZ) % NY), k = (int)(n % NZ);
        double acc[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 8; ++a) {
            int ei = i - ORC_CORNER[a][0], ej = j - ORC_CORNER[a][1], ek = k - ORC_CORNER[a][2];
            if (ei < 0 || ej < 0 || ek < 0 || ei >= nx || ej >= ny || ek >= nz) continue;
            double Ee = E[((int64_t)ei * ny + ej) * nz + ek];
            double pe[24];
            for (int b = 0; b < 8; ++b) {
                int64_t m = ((int64_t)(ei + ORC_CORNER[b][0]) * NY + (ej + ORC_CORNER[b][1])) * NZ +
                            (ek + ORC_CORNER[b][2]);
                for (int c = 0; c < 3; ++c)
                    pe[3 * b + c] = (fixed && fixed[3 * m + c]) ? 0.0 : p[3 * m + c];
            }
            for (int c = 0; c < 3; ++c) {
                const double *row = ke + (3 * a + c) * 24;
                double s = 0.0;
                for (int q = 0; q < 24; ++q) s += row[q] * pe[q];
                acc[c] += Ee * s;
            }
        }
        for (int c = 0; c < 3; ++c) y[3 * n + c] = (fixed && fixed[3 * n + c]) ? 0.0 : acc[c];
    }
}

/* Diagonal of D K(x) D (1 on fixed DOFs, so that the Jacobi step leaves them at 0 r). */
void orc_diag(int nx, int ny, int nz, const double *ke, const double *E, const uint8_t *fixed,
              double *dg) {
    const int64_t NY = ny + 1, NZ = nz + 1;
    const int64_t n_nodes = (int64_t)(nx + 1) * NY * NZ;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < n_nodes; ++n) {
        int i = (int)(n / (NY * NZ)), j = (int)((n / NZ) % NY), k = (int)(n % NZ);
        double acc[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 8; ++a) {
            int ei = i - ORC_CORNER[a][0], ej = j - ORC_CORNER[a][1], ek = k - ORC_CORNER[a][2];
            if (ei < 0 || ej < 0 || ek < 0 || ei >= nx || ej >= ny || ek >= nz) continue;
            double Ee = E[((int64_t)ei * ny + ej) * nz + ek];
            for (int c = 0; c < 3; ++c) acc[c] += Ee * ke[(3 * a + c) * 25];
        }
        for (int c = 0; c < 3; ++c) dg[3 * n + c] = (fixed && fixed[3 * n + c]) ? 1.0 : acc[c];
    }
}

/* ce_e = u_e^T Ke u_e and dc_e = -dE/dx(x_e) ce_e (simp_solver.py:215-218); returns
 * sum_e E_e ce_e = u^T K u. ce and dc are nullable. */
double orc_element_energy(int nx, int ny, int nz, const double *ke, const double *x,
                          const double *u, int law, double penal, double e0, double emin,
                          double xmin, double *ce, double *dc) {
    const int64_t NY = ny + 1, NZ = nz + 1;
    const int64_t n_elem = (int64_t)nx * ny * nz;
    double total = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : total)
    for (int64_t e = 0; e < n_elem; ++e) {
        int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double ue[24];
        for (int b = 0; b < 8; ++b) {
            int64_t m = ((int64_t)(i + ORC_CORNER[b][0]) * NY + (j + ORC_CORNER[b][1])) * NZ +
                        (k + ORC_CORNER[b][2]);
            for (int c = 0; c < 3; ++c) ue[3 * b + c] = u[3 * m + c];
        }
        double s = 0.0;
        for (int r = 0; r < 24; ++r) {
            double t = 0.0;
            for (int q = 0; q < 24; ++q) t += ke[r * 24 + q] * ue[q];
            s += ue[r] * t;
        }
        if (ce) ce[e] = s;
        if (dc) dc[e] = -orc_dE(law, x[e], penal, e0, emin, xmin) * s;
        total += orc_E(law, x[e], penal, e0, emin, xmin) * s;
    }
    return total;
}

/* Filter weights: H[e1,e2] = rmin - dist for dist <= rmin over the clipped box of
 * half-width ceil(rmin) (simp_solver.py:1545-1567); Hs = row sums. */
void orc_filter_hs(int nx, int ny, int nz, double rmin, double *hs) {
    const int r = (int)ceil(rmin);
    const int64_t n_elem = (int64_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n_elem; ++e) {
        int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double s = 0.0;
        for (int i2 = (i - r > 0 ? i - r : 0); i2 < (i + r + 1 < nx ? i + r + 1 : nx); ++i2)
            for (int j2 = (j - r > 0 ? j - r : 0); j2 < (j + r + 1 < ny ? j + r + 1 : ny); ++j2)
                for (int k2 = (k - r > 0 ? k - r : 0); k2 < (k + r + 1 < nz ? k + r + 1 : nz); ++k2) {
                    double d = sqrt((double)((i - i2) * (i - i2) + (j - j2) * (j - j2) + (k - k2) * (k - k2)));
                    if (d <= rmin) s += rmin - d;
                }
        hs[e] = s;
    }
}

/* transpose == 0: out = (H v) / Hs          (density filter, simp_solver.py:237)
 * transpose != 0: out = H^T (v / Hs)        (chain rule, simp_solver.py:221-223)
 * H is symmetric, so H^T (v/Hs) is a gather of v/Hs with the same weights. */
void orc_filter(int nx, int ny, int nz, double rmin, const double *hs, const double *v,
                int transpose, double *out) {
    const int r = (int)ceil(rmin);
    const int64_t n_elem = (int64_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n_elem; ++e) {
        int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double s = 0.0;
        for (int i2 = (i - r > 0 ? i - r : 0); i2 < (i + r + 1 < nx ? i + r + 1 : nx); ++i2)
            for (int j2 = (j - r > 0 ? j - r : 0); j2 < (j + r + 1 < ny ? j + r + 1 : ny); ++j2)
                for (int k2 = (k - r > 0 ? k - r : 0); k2 < (k + r + 1 < nz ? k + r + 1 : nz); ++k2) {
                    double d = sqrt((double)((i - i2) * (i - i2) + (j - j2) * (j - j2) + (k - k2) * (k - k2)));
                    if (d <= rmin) {
                        int64_t e2 = ((int64_t)i2 * ny + j2) * nz + k2;
                        s += (rmin - d) * (transpose ? v[e2] / hs[e2] : v[e2]);
                    }
                }
        out[e] = transpose ? s : s / hs[e];
    }
}

/* OC bisection (simp_solver.py:225-249). Parameters of the CPU variant: l1=0, l2=1e9,
 * max_bisect=50, tol=1e-4, tol_eps=1e-12, sqrt_floor=1e-12, move=0.2. GPU variant
 * (simp_solver_gpu.py:801-841): l2 = 2*max(max(-dc),1) (pass l2 < 0 to request it),
 * max_bisect=30, tol=1e-5, tol_eps=1e-15, sqrt_floor=1e-15. preserved is nullable.
 * Returns the number of bisection steps taken; xnew/xphys hold the last trial. */
int orc_oc(int nx, int ny, int nz, double rmin, const double *hs, const double *x,
           const double *dc, const uint8_t *preserved, double volfrac, double move, double l1,
           double l2, int max_bisect, double tol, double tol_eps, double sqrt_floor,
           double *xnew, double *xphys) {
    const int64_t n = (int64_t)nx * ny * nz;
    if (l2 < 0.0) {
        double m = -INFINITY;
        for (int64_t e = 0; e < n; ++e) m = (-dc[e] > m) ? -dc[e] : m;
        l2 = 2.0 * (m > 1.0 ? m : 1.0);
    }
    int it = 0;
    for (it = 0; it < max_bisect; ++it) {
        double lmid = 0.5 * (l2 + l1);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < n; ++e) {
            double t = -dc[e] / lmid;
            t = t > sqrt_floor ? t : sqrt_floor;
            double v = x[e] * sqrt(t);
            v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
            double lo = x[e] - move, hi = x[e] + move;
            v = v < lo ? lo : v;
            v = v > hi ? hi : v;
            if (preserved && preserved[e]) v = 1.0;
            xnew[e] = v;
        }
        orc_filter(nx, ny, nz, rmin, hs, xnew, 0, xphys);
        if (preserved)
            for (int64_t e = 0; e < n; ++e)
                if (preserved[e]) xphys[e] = 1.0;
        if ((l2 - l1) / (l1 + l2 + tol_eps) < tol) {
            ++it;
            break;
        }
        double vol = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : vol)
        for (int64_t e = 0; e < n; ++e) vol += xphys[e];
        if (vol / (double)n > volfrac)
            l1 = lmid;
        else
            l2 = lmid;
    }
    return it;
}

static double orc_dot(int64_t n, const double *a, const double *b) {
    double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* Jacobi-PCG on the free DOFs (fixed DOFs held at 0), the loop of
 * simp_solver_gpu.py:328-379: r = b - K x0, r[fixed]=0, z = r/diag, stop ||r|| < tol ||b||
 * with b = f with its fixed entries zeroed. u holds x0 on entry and the solution on exit.
 * Returns the iteration count; *relres gets ||r|| / ||b||. */
int orc_pcg(int nx, int ny, int nz, const double *ke, const double *E, const double *f,
            const uint8_t *fixed, double *u, double tol, int max_iter, double *relres) {
    const int64_t nd = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    double *r = (double *)malloc(nd * sizeof(double));
    double *z = (double *)malloc(nd * sizeof(double));
    double *p = (double *)malloc(nd * sizeof(double));
    double *q = (double *)malloc(nd * sizeof(double));
    double *dg = (double *)malloc(nd * sizeof(double));
    orc_diag(nx, ny, nz, ke, E, fixed, dg);
    for (int64_t i = 0; i < nd; ++i)
        if (fixed && fixed[i]) u[i] = 0.0;
    orc_apply(nx, ny, nz, ke, E, u, fixed, q);
    double bb = 0.0;
    for (int64_t i = 0; i < nd; ++i) {
        double bi = (fixed && fixed[i]) ? 0.0 : f[i];
        bb += bi * bi;
        r[i] = bi - q[i];
    }
    double bnorm = sqrt(bb);
    int it = 0;
    double rr = orc_dot(nd, r, r);
    if (bnorm == 0.0) {
        memset(u, 0, nd * sizeof(double));
        rr = 0.0;
        bnorm = 1.0;
    } else if (sqrt(rr) >= tol * bnorm) {
        for (int64_t i = 0; i < nd; ++i) {
            z[i] = r[i] / dg[i];
            p[i] = z[i];
        }
        double rz = orc_dot(nd, r, z);
        for (it = 0; it < max_iter;) {
            orc_apply(nx, ny, nz, ke, E, p, fixed, q);
            double pq = orc_dot(nd, p, q);
            if (!(pq > 0.0)) break;
            double alpha = rz / pq;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < nd; ++i) {
                u[i] += alpha * p[i];
                r[i] -= alpha * q[i];
            }
            ++it;
            rr = orc_dot(nd, r, r);
            if (sqrt(rr) < tol * bnorm) break;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < nd; ++i) z[i] = r[i] / dg[i];
            double rz_new = orc_dot(nd, r, z);
            double beta = rz_new / rz;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < nd; ++i) p[i] = z[i] + beta * p[i];
            rz = rz_new;
        }
    }
    if (relres) *relres = sqrt(rr) / bnorm;
    free(r);
    free(z);
    free(p);
    free(q);
    free(dg);
    return it;
}

/* One OC iteration of SIMPSolver.run (simp_solver.py:68-71): solve K(xphys) u = f
 * (u is the warm start on entry), dc from (xphys, u), dc <- H^T(dc/Hs), OC update of x.
 * Returns the PCG iteration count; *compliance gets f.u. */
int orc_simp_step(int nx, int ny, int nz, const double *ke, int law, double penal, double e0,
                  double emin, double xmin, double rmin, const double *hs, const double *f,
                  const uint8_t *fixed, const uint8_t *preserved, double volfrac, double *x,
                  double *xphys, double *u, double tol, int max_iter, double *compliance,
                  double *dc_out) {
    const int64_t ne = (int64_t)nx * ny * nz;
    const int64_t nd = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    double *E = (double *)malloc(ne * sizeof(double));
    double *dc = (double *)malloc(ne * sizeof(double));
    double *dcf = (double *)malloc(ne * sizeof(double));
    double *xn = (double *)malloc(ne * sizeof(double));
    orc_moduli(ne, xphys, law, penal, e0, emin, xmin, E);
    double rel = 0.0;
    int its = orc_pcg(nx, ny, nz, ke, E, f, fixed, u, tol, max_iter, &rel);
    orc_element_energy(nx, ny, nz, ke, xphys, u, law, penal, e0, emin, xmin, NULL, dc);
    orc_filter(nx, ny, nz, rmin, hs, dc, 1, dcf);
    orc_oc(nx, ny, nz, rmin, hs, x, dcf, preserved, volfrac, 0.2, 0.0, 1e9, 50, 1e-4, 1e-12,
           1e-12, xn, xphys);
    memcpy(x, xn, ne * sizeof(double));
    if (compliance) *compliance = orc_dot(nd, f, u);
    if (dc_out) memcpy(dc_out, dcf, ne * sizeof(double));
    free(E);
    free(dc);
    free(dcf);
    free(xn);
    return its;
}

/* SIMPSolver.run (simp_solver.py:56-79): x = volfrac (preserved -> 1), n_iters OC
 * iterations, then the compliance f.u of a final solve on the last xphys. x, xphys, u are
 * outputs (u: the final displacement). Returns the total PCG iteration count. */
long orc_simp_run(int nx, int ny, int nz, const double *ke, int law, double penal, double e0,
                  double emin, double xmin, double rmin, const double *f, const uint8_t *fixed,
                  const uint8_t *preserved, double volfrac, int n_iters, double tol,
                  int max_iter, double *x, double *xphys, double *u, double *compliance) {
    const int64_t ne = (int64_t)nx * ny * nz;
    const int64_t nd = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    double *hs = (double *)malloc(ne * sizeof(double));
    orc_filter_hs(nx, ny, nz, rmin, hs);
    for (int64_t e = 0; e < ne; ++e) {
        x[e] = (preserved && preserved[e]) ? 1.0 : volfrac;
        xphys[e] = x[e];
    }
    memset(u, 0, nd * sizeof(double));
    long total = 0;
    for (int it = 0; it < n_iters; ++it)
        total += orc_simp_step(nx, ny, nz, ke, law, penal, e0, emin, xmin, rmin, hs, f, fixed,
                               preserved, volfrac, x, xphys, u, tol, max_iter, NULL, NULL);
    double *E = (double *)malloc(ne * sizeof(double));
    orc_moduli(ne, xphys, law, penal, e0, emin, xmin, E);
    double rel = 0.0;
    total += orc_pcg(nx, ny, nz, ke, E, f, fixed, u, tol, max_iter, &rel);
    if (compliance) *compliance = orc_dot(nd, f, u);
    free(E);
    free(hs);
    return total;
}
