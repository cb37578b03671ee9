/*
 * spectral_oracle.h -- CPU restatement of SpectralBTE's spectral-Lagrangian
 * collision path (reference: src/collisions.c, src/conserve.c,
 * src/momentRoutines.c, src/weights.c, src/initializer.c, exec/boltz.c).
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT.  Only tests/, the smoke check and the
 * CPU-baseline leg of bench.py may load this code, and only to check or
 * time against it.  The GPU library never calls it.
 *
 * Every routine takes its state explicitly, with no file-scope statics, so
 * the tests can run several grids side by side.  Each one cites the
 * reference lines whose arithmetic it restates.  Summation orders follow
 * the reference loops, so results agree with the reference to the last
 * bit given identical FFT outputs.
 *
 * Layouts (as in the reference):
 *   - a velocity or Fourier index (i,j,k) maps to k + N*(j + N*i),
 *     with i the slowest axis (collisions.c:99-102);
 *   - complex arrays are interleaved (re, im) pairs, like fftw_complex;
 *   - W is one row-major [N^3][N^3] array, row = zeta and column = xi
 *     (weights.c:277; the reference keeps it as an array of row pointers).
 */
#ifndef SPECTRAL_ORACLE_H
#define SPECTRAL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- grids ------------------------------------------------------------ */
/* 0D grid, initializer.c:66-82. */
void oracle_grid_0d(int N, double L_v, double *v, double *zeta);
/* 1D grid, initializer.c:256-266. */
void oracle_grid_1d(int N, double L_v, double *v, double *zeta);

/* ---- FFT with phase shift and trapezoid weights (collisions.c:232-283) -- */
/* in/out: interleaved complex N^3.  invert = 0 forward, 1 inverse.
   in and out may alias. */
void oracle_fft3d(int N, double L_v, const double *v, const double *zeta,
                  const double *in, double *out, int invert);

/* ---- weighted convolution (collisions.c:108-169) ---------------------- */
/* Computes the forward transforms of f and g and qhat[zeta] =
   sum_xi W[zeta][xi] ghat[xi] fhat[idx(zeta, xi)].  If q is non-NULL it
   also writes Re(inverse fft3D(qhat)).  fhat_out/ghat_out/qhat_out may be
   NULL. */
void oracle_compute_qhat(int N, double L_v, const double *v,
                         const double *zeta, const double *W,
                         const double *f, const double *g, double *q,
                         double *fhat_out, double *ghat_out,
                         double *qhat_out, int nthreads);

/* The inner loop of compute_Qhat (collisions.c:127-165) for zeta rows
   [row0, row0+nrows) only: qhat[zeta - row0] from precomputed transforms
   fhat, ghat (interleaved complex N^3) and W rows W[(zeta-row0)*N^3 + xi].
   Used to time a bounded sample of the convolution on the CPU. */
void oracle_qhat_rows(int N, const double *W_rows, int row0, int nrows,
                      const double *fhat, const double *ghat, double *qhat,
                      int nthreads);

/* ComputeQ (collisions.c:212-221). */
void oracle_computeQ(int N, double L_v, const double *v, const double *zeta,
                     const double *W, const double *f, const double *g,
                     double *Q, int nthreads);

/* ComputeQ_maxPreserve (collisions.c:178-210) with find_maxwellians
   (:91-106).  mass and KB are the momentRoutines.c parameters of species 0
   (momentRoutines.c:23-28). */
void oracle_computeQ_maxPreserve(int N, double L_v, const double *v,
                                 const double *zeta, const double *W,
                                 const double *f, const double *g, double *Q,
                                 double mass, double KB, int nthreads);

/* ---- moments (momentRoutines.c:58-69, 116-141, 168-183, 146-165) ------ */
double oracle_density(int N, const double *v, const double *f, double mass);
void oracle_bulk_velocity(int N, const double *v, const double *f, double rho,
                          double mass, double *u);
double oracle_temperature(int N, const double *v, const double *f,
                          const double *u, double rho, double mass, double KB);
void oracle_energy(int N, const double *v, const double *f, double *out2);

/* ---- conservation (conserve.c) ---------------------------------------- */
#define ORACLE_MAX_NS 4
typedef struct {
    int N, Ns;
    double dv;
    const double *v;
    double mass[ORACLE_MAX_NS];
    double CCt[ORACLE_MAX_NS + 4][ORACLE_MAX_NS + 4]; /* LU factors */
    int pivot[ORACLE_MAX_NS + 4];
} oracle_cons;

/* initialize_conservation + createCCtAndPivot + factorMatrixIntoLU
   (conserve.c:17-43, 268-317, 89-168).  Returns 0, or -1 when the matrix
   is singular (the reference calls exit(0), conserve.c:130-135). */
int oracle_conservation_init(oracle_cons *c, int N, double dv,
                             const double *v, const double *mass, int Ns);
/* solveWithCCt (conserve.c:173-202); b has Ns+4 entries, solved in place. */
void oracle_solve_cct(const oracle_cons *c, double *b);
/* conserveAllMoments (conserve.c:207-264); Q[n*Ns+m] are N^3 arrays. */
void oracle_conserve(const oracle_cons *c, double **Q);
/* Same, but for one species and a flat batch of B arrays of N^3. */
void oracle_conserve_batch1(const oracle_cons *c, double *Q, int B);

/* ---- weight quadrature (weights.c:44, 136-160, 181-281) ---------------- */
/* Gauss-Legendre nodes and weights on [-1,1] (n <= 256). */
void oracle_gauss_legendre(int n, double *x, double *w);
double oracle_ghat3l(double zeta1, double zeta2, double zeta3, double xi1, double xi2,
                     double xi3, double L_v, double lambda);
void oracle_weights_landau(int N, const double *eta, double L_v, double lambda, int row0,
                           int nrows, double *W);
/* Grazing-collision weights of the stand-alone generator
   (MPIcollisionRoutines.c:33-205), composite Gauss-Legendre at every level
   (spectral_oracle.c): theta panel edges (returns the panel count), the r and
   phi panel count for a grid with max |eta| = L_eta, one weight, and a list
   of (zeta, xi) pairs. */
int oracle_graze_theta_edges(double glance, double *edges);
int oracle_graze_panels(double L_eta, double L_v);
double oracle_ghat3_graze(double zeta1, double zeta2, double zeta3, double xi1, double xi2,
                          double xi3, double L_v, double lambda, double glance, int npan);
void oracle_ghat3_graze_pairs(int npairs, const double *pairs, double L_v, double lambda,
                              double glance, int npan, double *out);
/* Number of 16-point Gauss-Legendre panels the oracle uses on [0, L_v] for an
   integrand whose highest angular frequency is omega. */
int oracle_quad_panels(double L_v, double omega);
/* gHat3 without the prefactor: integral over [0, L_v] of
   r^(lambda+2) [sinc(r a0) sinc(r a2) - sinc(r a1)] dr,
   a0 = mu|zeta|, a1 = |ki|, a2 = |ki - mu zeta|, mu = m_j / (m_i + m_j). */
double oracle_ghat_integral(double a0, double a1, double a2, double lambda,
                            double L_v);
/* Rows [row_begin, row_end) of the isotropic weights
   W[zeta=(i,j,k)][xi=(l,m,n)] (weights.c:265-281), written to
   W[(row - row_begin) * N^3 + col]. */
void oracle_weights_iso(int N, const double *zeta, double L_v, double lambda,
                        double d_i, double d_j, double m_i, double m_j,
                        int row_begin, int row_end, double *W, int nthreads);
/* The same integral in closed form for lambda = 0 and 1 (quadrature for
   other lambda and for nonzero gain arguments below 1/(2 L_v)), and the
   weights built from it. */
double oracle_ghat_closed(double a0, double a1, double a2, double lambda, double L_v);
void oracle_weights_iso_closed(int N, const double *zeta, double L_v, double lambda,
                               double d_i, double d_j, double m_i, double m_j,
                               int row_begin, int row_end, double *W, int nthreads);

/* ---- 0D driver (exec/boltz.c:186-250, output.c:159-213) ---------------- */
/* Runs nT steps of the homogeneous solver for one species with the
   maxPreserve operator (boltz.c:196), conservation and order-1 (Euler) or
   order-2 (RK2) updates.  Row t of rows (t = 0..nT, stride 6 + N) holds
   time, density, u_x, temperature, pressure, energy ratio and the slice
   f[N/2 + N*(N/2 + N*l)]; these are the columns write_streams prints. */
void oracle_run_0d(int N, double L_v, const double *W, double *f, double dt,
                   double Kn, int nT, int order, int maxpreserve,
                   double *rows, int nthreads);

/* BKW initial data, initializer.c:123-135 (K from t0 = 5.5 unless K > 0). */
void oracle_init_bkw(int N, const double *v, double K, double *f);

/* ---- 1D driver (exec/boltz.c:254-394, transportroutines.c,
        boundaryConditions.c, initializer.c:296-424, mesh_setup.c) ------- */
typedef struct {
    int N, nX, order, ic;      /* ic = the reference's Init_field value */
    double L_v, dt, Kn;
    double T0, T1, TWall;      /* wall temperatures (transportroutines.c:46-50) */
    double mass, KB;
    const double *x, *dx;      /* nX + 2*order entries incl. ghost cells */
} oracle_1d;

/* One zone of nX cells over [0, length], single rank (mesh_setup.c:59-160),
   ghost cells by uniform extension on both sides. */
void oracle_mesh_uniform(int nX, double length, int order, double *x, double *dx);
/* Initial data of the interior cells, initializer.c:296-424. f holds
   nX + 2*order cells of N^3. */
void oracle_init_1d(const oracle_1d *p, const double *v, double *f);
/* Diffuse reflection, boundaryConditions.c:39-96 (bdry 0 = left wall). */
void oracle_diffuse_bc(int N, const double *v, const double *in, double *out,
                       double TW, int bdry, double mass, double KB);
/* upwindOne / advectTwo for a single rank (transportroutines.c:94-238,
   241-470, 477-492).  f and fconv hold nX + 2*order cells.  scratch holds
   nX + 2*order + 2 cells. */
void oracle_advect(const oracle_1d *p, const double *v, double *f, double *fconv,
                   double *scratch);
/* nT steps of the 1D loop (boltz.c:264-394) with ComputeQ + conservation per
   cell; rows receives (nT+1) dumps of nX lines (time, x, density, u_x,
   temperature, pressure), as write_streams_inhom prints (output.c:295-340). */
void oracle_run_1d(const oracle_1d *p, const double *W, double *f, int nT,
                   double *rows, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
