/*
 * swalbe_oracle.c -- CPU oracle for the thin-film LBM time step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file.  Only tests/, __graft_entry__.smoke() and bench.py (its
 * CPU-baseline leg and its `--impl reference` arm) use it, as the checker.
 *
 * The reference (Swalbe.jl) is pure Julia; Julia is not available here, so
 * this file restates the reference's Float64 algorithm in C.  Two layers:
 *
 *   1. a LITERAL restatement: one loop per Julia `.=` broadcast statement,
 *      the same left-to-right association, `circshift!` materialised into the
 *      same `dgrad` planes, compiled with -ffp-contract=off (Julia does not
 *      contract a*b+c into FMA).  Each function cites the reference line it
 *      follows (paths relative to the Swalbe.jl project root).
 *
 *   2. a FUSED restatement (orc_fused_run) that performs exactly the same
 *      per-cell floating-point operations in three OpenMP passes per step
 *      over a post-collision ("pull") population buffer.  It is bit-identical
 *      to layer 1 (checked by tests) and is the timed CPU baseline.
 *
 * Layout: every field is column-major, x (i) fastest, exactly as Julia stores
 * `zeros(Lx, Ly)`; populations are 9 planes `f[i,j,q]` (src/initialize.jl:493).
 *
 * Pinning: the unit golden vectors of the reference test-suite (test/*.jl)
 * and its doctests are checked against these functions in
 * tests/test_oracle_golden.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(i, j, Lx) ((size_t)(i) + (size_t)(Lx) * (size_t)(j))

static inline int wrapi(int i, int L) {
    int r = i % L;
    return r < 0 ? r + L : r;
}

/* ------------------------------------------------------------------ */
/* Parameters: mirror of Taumucs{T} + SysConst{T}                      */
/* (src/initialize.jl:43-60, 76-81).  Same layout as swb_params in     */
/* include/swalbe_gb300.h so that the Python side can share one struct. */
/* ------------------------------------------------------------------ */
typedef struct {
    int32_t Lx, Ly;
    int32_t Tmax, tdump;
    double tau, cs, mu, delta, kbt, gamma;
    int32_t n, m;
    double hmin, hcrit, theta, g;
} orc_params;

/* cospi(x) = cos(pi x); exact at multiples of 1/2 like Julia's Base.cospi,
 * otherwise evaluated in long double and rounded once. */
double orc_cospi(double x) {
    if (!isfinite(x)) return NAN;
    double r = fmod(fabs(x), 2.0); /* exact */
    if (r == 0.0) return 1.0;
    if (r == 1.0) return -1.0;
    if (r == 0.5 || r == 1.5) return 0.0;
    const long double PI_L = 3.141592653589793238462643383279502884L;
    return (double)cosl(PI_L * (long double)r);
}

/* circshift!(dst, src, (a, b)): dst[i,j] = src[mod1(i-a), mod1(j-b)] (Julia Base) */
void orc_circshift(double *dst, const double *src, int Lx, int Ly, int a, int b) {
    for (int j = 0; j < Ly; ++j)
        for (int i = 0; i < Lx; ++i)
            dst[IDX(i, j, Lx)] = src[IDX(wrapi(i - a, Lx), wrapi(j - b, Ly), Lx)];
}

/* The 8 neighbour planes in viewneighbors order (src/differences.jl:251-262),
 * filled with the shifts used by filmpressure!, h∇p! and ∇f!. */
static void neighbours(double *dgrad, const double *f, int Lx, int Ly) {
    size_t N = (size_t)Lx * Ly;
    orc_circshift(dgrad + 0 * N, f, Lx, Ly, 1, 0);   /* ip   */
    orc_circshift(dgrad + 1 * N, f, Lx, Ly, 0, 1);   /* jp   */
    orc_circshift(dgrad + 2 * N, f, Lx, Ly, -1, 0);  /* im   */
    orc_circshift(dgrad + 3 * N, f, Lx, Ly, 0, -1);  /* jm   */
    orc_circshift(dgrad + 4 * N, f, Lx, Ly, 1, 1);   /* ipjp */
    orc_circshift(dgrad + 5 * N, f, Lx, Ly, -1, 1);  /* imjp */
    orc_circshift(dgrad + 6 * N, f, Lx, Ly, -1, -1); /* imjm */
    orc_circshift(dgrad + 7 * N, f, Lx, Ly, 1, -1);  /* ipjm */
}

/* power_broad(arg, n): repeated multiplication from 1.0 (src/pressure.jl:363-369) */
double orc_power_broad(double x, int n) {
    double t = 1.0;
    for (int i = 0; i < n; ++i) t *= x;
    return t;
}
static inline double power_3(double x) { return x * x * x; } /* src/pressure.jl:401-403 */
static inline double fast_93(double x) {                     /* src/pressure.jl:410-413 */
    double t = power_3(x);
    return power_3(t) - t;
}
static inline double fast_32(double x) { return power_3(x) - x * x; } /* src/pressure.jl:420-422 */

/* kappa prefactor (((1 - cospi θ)(n-1))(m-1)) / ((n-m) hmin), evaluated in
 * the broadcast's left-to-right order (src/pressure.jl:141-147). */
double orc_kappa(double theta, int n, int m, double hmin) {
    double a = 1.0 - orc_cospi(theta);
    a = a * (double)(n - 1);
    a = a * (double)(m - 1);
    return a / ((double)(n - m) * hmin);
}

/* Laplacian part shared by filmpressure! (pressure.jl:149-153) and ∇²f!
 * (differences.jl:69-73): 2/3 Σ straight + 1/6 Σ diagonal - 10/3 f */
static inline double lap9(const double *d, size_t N, size_t k, double fk) {
    const double *ip = d, *jp = d + N, *im = d + 2 * N, *jm = d + 3 * N;
    const double *ipjp = d + 4 * N, *imjp = d + 5 * N, *imjm = d + 6 * N, *ipjm = d + 7 * N;
    return (2.0 / 3.0) * (((jp[k] + ip[k]) + im[k]) + jm[k]) +
           (1.0 / 6.0) * (((ipjp[k] + imjp[k]) + imjm[k]) + ipjm[k]) - (10.0 / 3.0) * fk;
}

/* filmpressure!(state, sys; θ) -- state form with power_broad
 * (src/pressure.jl:119-155).  theta_field may be NULL (scalar θ). */
void orc_filmpressure(double *p, const double *h, double *dgrad, int Lx, int Ly, double gamma,
                      const double *theta_field, double theta, int n, int m, double hmin,
                      double hcrit) {
    size_t N = (size_t)Lx * Ly;
    neighbours(dgrad, h, Lx, Ly);
    double kap_s = orc_kappa(theta, n, m, hmin);
    for (size_t k = 0; k < N; ++k) {
        double kap = theta_field ? orc_kappa(theta_field[k], n, m, hmin) : kap_s;
        double x = hmin / (h[k] + hcrit);
        p[k] = -gamma * (kap * (orc_power_broad(x, n) - orc_power_broad(x, m)));
    }
    for (size_t k = 0; k < N; ++k) p[k] = p[k] - gamma * lap9(dgrad, N, k, h[k]);
}

/* filmpressure!(output, f, dgrad, γ, θ, n, m, hmin, hcrit) -- the raw form
 * with fast_93 / fast_32 (src/pressure.jl:72-115).  Returns -1 for exponent
 * pairs other than (9,3) and (3,2), where the reference throws DomainError. */
int orc_filmpressure_raw(double *p, const double *h, double *dgrad, int Lx, int Ly, double gamma,
                         double theta, int n, int m, double hmin, double hcrit) {
    size_t N = (size_t)Lx * Ly;
    if (!((n == 9 && m == 3) || (n == 3 && m == 2))) return -1;
    neighbours(dgrad, h, Lx, Ly);
    double kap = orc_kappa(theta, n, m, hmin);
    for (size_t k = 0; k < N; ++k) {
        double x = hmin / (h[k] + hcrit);
        double v = (n == 9) ? fast_93(x) : fast_32(x);
        p[k] = -gamma * (kap * v);
    }
    for (size_t k = 0; k < N; ++k) p[k] = p[k] - gamma * lap9(dgrad, N, k, h[k]);
    return 0;
}

/* ∇²f!(output, f, γ) (src/differences.jl:57-75) */
void orc_laplacian(double *out, const double *f, double *dgrad, int Lx, int Ly, double gamma) {
    size_t N = (size_t)Lx * Ly;
    neighbours(dgrad, f, Lx, Ly);
    for (size_t k = 0; k < N; ++k) out[k] = gamma * lap9(dgrad, N, k, f[k]);
}

/* Gradient stencil of ∇f! / ∇f_simple! (src/differences.jl:165-166,
 * src/measures.jl:188-189). */
static inline void grad9(const double *d, size_t N, size_t k, double *gx, double *gy) {
    const double *ip = d, *jp = d + N, *im = d + 2 * N, *jm = d + 3 * N;
    const double *ipjp = d + 4 * N, *imjp = d + 5 * N, *imjm = d + 6 * N, *ipjm = d + 7 * N;
    *gx = (-1.0 / 3.0) * (ip[k] - im[k]) - (1.0 / 12.0) * (((ipjp[k] - imjp[k]) - imjm[k]) + ipjm[k]);
    *gy = (-1.0 / 3.0) * (jp[k] - jm[k]) - (1.0 / 12.0) * (((ipjp[k] + imjp[k]) - imjm[k]) - ipjm[k]);
}

/* ∇f!(outputx, outputy, f) (src/differences.jl:153-169) */
void orc_gradient(double *gx, double *gy, const double *f, double *dgrad, int Lx, int Ly) {
    size_t N = (size_t)Lx * Ly;
    neighbours(dgrad, f, Lx, Ly);
    for (size_t k = 0; k < N; ++k) grad9(dgrad, N, k, &gx[k], &gy[k]);
}

/* h∇p!(state) (src/forcing.jl:168-187) */
void orc_hgradp(double *hgx, double *hgy, const double *h, const double *p, double *dgrad, int Lx,
                int Ly) {
    size_t N = (size_t)Lx * Ly;
    neighbours(dgrad, p, Lx, Ly);
    const double *fip = dgrad, *fjp = dgrad + N, *fim = dgrad + 2 * N, *fjm = dgrad + 3 * N;
    const double *fipjp = dgrad + 4 * N, *fimjp = dgrad + 5 * N, *fimjm = dgrad + 6 * N,
                 *fipjm = dgrad + 7 * N;
    for (size_t k = 0; k < N; ++k)
        hgx[k] = h[k] * ((-1.0 / 3.0) * (fip[k] - fim[k]) -
                         (1.0 / 12.0) * (((fipjp[k] - fimjp[k]) - fimjm[k]) + fipjm[k]));
    for (size_t k = 0; k < N; ++k)
        hgy[k] = h[k] * ((-1.0 / 3.0) * (fjp[k] - fjm[k]) -
                         (1.0 / 12.0) * (((fipjp[k] + fimjp[k]) - fimjm[k]) - fipjm[k]));
}

/* slippage!(slipx, slipy, height, velx, vely, δ, μ) (src/forcing.jl:42-46) */
void orc_slippage(double *sx, double *sy, const double *h, const double *ux, const double *uy,
                  size_t N, double delta, double mu) {
    for (size_t k = 0; k < N; ++k)
        sx[k] = ((6.0 * mu) * h[k] * ux[k]) /
                (2.0 * (h[k] * h[k]) + (6.0 * delta) * h[k] + 3.0 * (delta * delta));
    for (size_t k = 0; k < N; ++k)
        sy[k] = ((6.0 * mu) * h[k] * uy[k]) /
                (2.0 * (h[k] * h[k]) + (6.0 * delta) * h[k] + 3.0 * (delta * delta));
}

/* Fx .= -h∇px .- slipx ; Fy likewise (src/simulate.jl:18-19) */
void orc_force_sum(double *Fx, double *Fy, const double *hgx, const double *hgy, const double *sx,
                   const double *sy, size_t N) {
    for (size_t k = 0; k < N; ++k) Fx[k] = -hgx[k] - sx[k];
    for (size_t k = 0; k < N; ++k) Fy[k] = -hgy[k] - sy[k];
}

/* The smoothing factor of inclination!: 0.5 + 0.5 tanh((t - tstart)/tsmooth) */
double orc_incl_factor(long t, long tstart, long tsmooth) {
    return 0.5 + 0.5 * tanh((double)(t - tstart) / (double)tsmooth);
}

/* inclination!(α, state; t, tstart, tsmooth) (src/forcing.jl:363-368) */
void orc_inclination(double *Fx, double *Fy, const double *h, size_t N, double ax, double ay,
                     long t, long tstart, long tsmooth) {
    double s = orc_incl_factor(t, tstart, tsmooth);
    for (size_t k = 0; k < N; ++k) Fx[k] = Fx[k] + (h[k] * ax) * s;
    for (size_t k = 0; k < N; ++k) Fy[k] = Fy[k] + (h[k] * ay) * s;
}

/* One cell of equilibrium! (src/equilibrium.jl:63-116); vsq is returned. */
static inline double feq_cell(double h, double ux, double uy, double g, double fe[9]) {
    const double g0 = 1.5 * g, w1 = 1.0 / 9.0, w5 = 1.0 / 36.0;
    double vsq = ux * ux + uy * uy;
    fe[0] = h * ((1.0 - (5.0 / 6.0) * g * h) - (2.0 / 3.0) * vsq);
    fe[1] = w1 * h * (g0 * h + 3.0 * ux + 4.5 * (ux * ux) - 1.5 * vsq);
    fe[2] = w1 * h * (g0 * h + 3.0 * uy + 4.5 * (uy * uy) - 1.5 * vsq);
    fe[3] = w1 * h * (g0 * h - 3.0 * ux + 4.5 * (ux * ux) - 1.5 * vsq);
    fe[4] = w1 * h * (g0 * h - 3.0 * uy + 4.5 * (uy * uy) - 1.5 * vsq);
    fe[5] = w5 * h * (g0 * h + 3.0 * (ux + uy) + 4.5 * ((ux + uy) * (ux + uy)) - 1.5 * vsq);
    fe[6] = w5 * h * (g0 * h + 3.0 * (uy - ux) + 4.5 * ((uy - ux) * (uy - ux)) - 1.5 * vsq);
    fe[7] = w5 * h * (g0 * h - 3.0 * (ux + uy) + 4.5 * ((ux + uy) * (ux + uy)) - 1.5 * vsq);
    fe[8] = w5 * h * (g0 * h + 3.0 * (ux - uy) + 4.5 * ((ux - uy) * (ux - uy)) - 1.5 * vsq);
    return vsq;
}

/* equilibrium!(feq, height, velx, vely, vsq, g) (src/equilibrium.jl:63-116).
 * The reference evaluates one plane after another; each plane's value per
 * cell only depends on (h, ux, uy, vsq), so the per-cell loop is identical. */
void orc_equilibrium(double *feq, const double *h, const double *ux, const double *uy, double *vsq,
                     size_t N, double g) {
    double fe[9];
    for (size_t k = 0; k < N; ++k) {
        vsq[k] = feq_cell(h[k], ux[k], uy[k], g, fe);
        for (int q = 0; q < 9; ++q) feq[q * N + k] = fe[q];
    }
}

/* D2Q9 lattice velocities in the reference's order (src/collide.jl:92-100) */
static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

/* One cell of the BGK collision with the force source (src/collide.jl:76-89). */
static inline void collide_cell(const double ft[9], const double fe[9], double Fx, double Fy,
                                double omeg, double invtau, double fo[9]) {
    fo[0] = omeg * ft[0] + invtau * fe[0];
    fo[1] = omeg * ft[1] + invtau * fe[1] + (1.0 / 3.0) * Fx;
    fo[2] = omeg * ft[2] + invtau * fe[2] + (1.0 / 3.0) * Fy;
    fo[3] = omeg * ft[3] + invtau * fe[3] - (1.0 / 3.0) * Fx;
    fo[4] = omeg * ft[4] + invtau * fe[4] - (1.0 / 3.0) * Fy;
    fo[5] = omeg * ft[5] + invtau * fe[5] + (1.0 / 24.0) * (Fx + Fy);
    fo[6] = omeg * ft[6] + invtau * fe[6] + (1.0 / 24.0) * (Fy - Fx);
    fo[7] = omeg * ft[7] + invtau * fe[7] - (1.0 / 24.0) * (Fx + Fy);
    fo[8] = omeg * ft[8] + invtau * fe[8] + (1.0 / 24.0) * (Fx - Fy);
}

/* BGKandStream!(fout, feq, ftemp, Fx, Fy, τ) (src/collide.jl:70-105):
 * collide into fout, stream fout into ftemp by circshift!, copy back. */
void orc_bgk_stream(double *fout, const double *feq, double *ftemp, const double *Fx,
                    const double *Fy, int Lx, int Ly, double tau) {
    size_t N = (size_t)Lx * Ly;
    double omeg = 1.0 - 1.0 / tau, invtau = 1.0 / tau;
    double ft[9], fe[9], fo[9];
    for (size_t k = 0; k < N; ++k) {
        for (int q = 0; q < 9; ++q) {
            ft[q] = ftemp[q * N + k];
            fe[q] = feq[q * N + k];
        }
        collide_cell(ft, fe, Fx[k], Fy[k], omeg, invtau, fo);
        for (int q = 0; q < 9; ++q) fout[q * N + k] = fo[q];
    }
    for (int q = 0; q < 9; ++q) orc_circshift(ftemp + q * N, fout + q * N, Lx, Ly, CX[q], CY[q]);
    memcpy(fout, ftemp, 9 * N * sizeof(double));
}

/* moments!(height, velx, vely, fout) (src/moments.jl:43-51): sum! over the
 * third dimension accumulates q = 1..9 in order starting from zero. */
static inline void moments_cell(const double f[9], double *h, double *ux, double *uy) {
    double s = 0.0;
    for (int q = 0; q < 9; ++q) s = s + f[q];
    *h = s;
    *ux = (f[1] - f[3] + f[5] - f[6] - f[7] + f[8]) / s;
    *uy = (f[2] - f[4] + f[5] + f[6] - f[7] - f[8]) / s;
}

void orc_moments(double *h, double *ux, double *uy, const double *fout, size_t N) {
    double f[9];
    for (size_t k = 0; k < N; ++k) {
        for (int q = 0; q < 9; ++q) f[q] = fout[q * N + k];
        moments_cell(f, &h[k], &ux[k], &uy[k]);
    }
}

/* ------------------------------------------------------------------ */
/* Measures (src/measures.jl, src/simulate.jl:10,56)                    */
/* ------------------------------------------------------------------ */

/* Pairwise summation with a 1024-element base case; the reference's sum()
 * is also pairwise (Base.mapreduce_impl), so both have O(log N) error. */
static double pairwise_sum(const double *a, size_t n) {
    if (n <= 1024) {
        long double s = 0.0L;
        for (size_t k = 0; k < n; ++k) s += a[k];
        return (double)s;
    }
    size_t h = n / 2;
    return pairwise_sum(a, h) + pairwise_sum(a + h, n - h);
}

double orc_sum(const double *a, size_t N) { return pairwise_sum(a, N); }

/* wetted!(area, state): length(findall(h .> hthresh)) (src/measures.jl:13-17) */
int64_t orc_wetted(const double *h, size_t N, double hthresh) {
    int64_t c = 0;
    for (size_t k = 0; k < N; ++k) c += (h[k] > hthresh);
    return c;
}

/* maximum(h) - minimum(h) (src/simulate.jl:56) */
double orc_dh(const double *h, size_t N) {
    double mx = h[0], mn = h[0];
    for (size_t k = 1; k < N; ++k) {
        if (h[k] > mx) mx = h[k];
        if (h[k] < mn) mn = h[k];
    }
    return mx - mn;
}

/* surfacearea!(area_lv, red_energy, height, θ, ...) (src/measures.jl:126-168)
 * with ∇f_simple! (src/measures.jl:175-192).  theta_field may be NULL. */
void orc_surfacearea(const double *h, const double *theta_field, double theta, int Lx, int Ly,
                     double htresh, double *dgrad, double *area_out, double *energy_out) {
    size_t N = (size_t)Lx * Ly;
    neighbours(dgrad, h, Lx, Ly);
    long double surf = 0.0L, cossum = 0.0L;
    int64_t nwet = 0;
    for (size_t k = 0; k < N; ++k) {
        if (!(h[k] > htresh)) continue;
        double gx, gy;
        grad9(dgrad, N, k, &gx, &gy);
        surf += sqrt(gx * gx + gy * gy + 1.0);
        if (theta_field) cossum += orc_cospi(theta_field[k]);
        nwet++;
    }
    *area_out = (double)surf;
    if (theta_field)
        *energy_out = (double)surf - (double)cossum;
    else
        *energy_out = (double)surf - (double)nwet * orc_cospi(theta);
}

/* ------------------------------------------------------------------ */
/* Initial values (src/initialvalues.jl)                                */
/* ------------------------------------------------------------------ */

/* singledroplet(height, radius, θ, center) (src/initialvalues.jl:203-224);
 * center is 1-based like the reference. */
void orc_singledroplet(double *h, int Lx, int Ly, double radius, double theta, double cx,
                       double cy) {
    double c = orc_cospi(theta);
    for (int i = 1; i <= Lx; ++i)
        for (int j = 1; j <= Ly; ++j) {
            double di = (double)i - cx, dj = (double)j - cy;
            double circ = sqrt(di * di + dj * dj);
            double v;
            if (circ <= radius)
                v = (cos(asin(circ / radius)) - c) * radius;
            else
                v = 0.05;
            h[IDX(i - 1, j - 1, Lx)] = v;
        }
    for (size_t k = 0; k < (size_t)Lx * Ly; ++k)
        if (h[k] < 0) h[k] = 0.05;
}

/* ------------------------------------------------------------------ */
/* LITERAL state + time_loop (src/initialize.jl:149-168, 491-508;       */
/* src/simulate.jl:6-96)                                                */
/* ------------------------------------------------------------------ */
typedef struct {
    int Lx, Ly;
    double *fout, *ftemp, *feq;                    /* 9N each */
    double *height, *velx, *vely, *vsq, *pressure; /* N each */
    double *Fx, *Fy, *slipx, *slipy, *hgx, *hgy;   /* N each */
    double *dgrad;                                 /* 8N */
} orc_state;

/* Sys(sysc, "CPU"): zeros everywhere, height = 1 (src/initialize.jl:491-508) */
orc_state *orc_state_new(int Lx, int Ly) {
    size_t N = (size_t)Lx * Ly;
    orc_state *s = (orc_state *)calloc(1, sizeof(orc_state));
    if (!s) return NULL;
    s->Lx = Lx;
    s->Ly = Ly;
    s->fout = (double *)calloc(9 * N, sizeof(double));
    s->ftemp = (double *)calloc(9 * N, sizeof(double));
    s->feq = (double *)calloc(9 * N, sizeof(double));
    s->height = (double *)calloc(N, sizeof(double));
    s->velx = (double *)calloc(N, sizeof(double));
    s->vely = (double *)calloc(N, sizeof(double));
    s->vsq = (double *)calloc(N, sizeof(double));
    s->pressure = (double *)calloc(N, sizeof(double));
    s->Fx = (double *)calloc(N, sizeof(double));
    s->Fy = (double *)calloc(N, sizeof(double));
    s->slipx = (double *)calloc(N, sizeof(double));
    s->slipy = (double *)calloc(N, sizeof(double));
    s->hgx = (double *)calloc(N, sizeof(double));
    s->hgy = (double *)calloc(N, sizeof(double));
    s->dgrad = (double *)calloc(8 * N, sizeof(double));
    for (size_t k = 0; k < N; ++k) s->height[k] = 1.0;
    return s;
}

void orc_state_free(orc_state *s) {
    if (!s) return;
    free(s->fout); free(s->ftemp); free(s->feq);
    free(s->height); free(s->velx); free(s->vely); free(s->vsq); free(s->pressure);
    free(s->Fx); free(s->Fy); free(s->slipx); free(s->slipy); free(s->hgx); free(s->hgy);
    free(s->dgrad);
    free(s);
}

/* Field access for the Python harness.  ids: 0 fout, 1 ftemp, 2 feq,
 * 3 height, 4 velx, 5 vely, 6 vsq, 7 pressure, 8 Fx, 9 Fy, 10 slipx,
 * 11 slipy, 12 h∇px, 13 h∇py, 14 dgrad. */
double *orc_state_field(orc_state *s, int id) {
    double *t[15] = {s->fout,     s->ftemp, s->feq, s->height, s->velx,
                     s->vely,     s->vsq,   s->pressure, s->Fx, s->Fy,
                     s->slipx,    s->slipy, s->hgx, s->hgy, s->dgrad};
    return (id >= 0 && id < 15) ? t[id] : NULL;
}

/* Loop options shared by the literal and the fused time loops. */
typedef struct {
    const double *theta_field; /* NULL: scalar θ (time_loop(sys, state[, θ])) */
    double theta;              /* scalar θ used when theta_field is NULL       */
    int record_dh;             /* time_loop(sys, state, Δh) (simulate.jl:56)   */
    int callback;              /* 0 none, 1 wetted!, 2 inclination!            */
    double hthresh;            /* wetted! threshold, 0.055                     */
    double incl_ax, incl_ay;   /* inclination! α                                */
    int incl_loop_time;        /* 1: t = loop iteration, 0: t = incl_t        */
    long incl_t, incl_tstart, incl_tsmooth;
    uint64_t thermal_seed;     /* thermal! noise stream (used when kbt > 0)     */
    long t_offset;             /* iterations done before this call (noise index) */
    long shift_tmove;          /* moving θ field: move_substrate! every tmove     */
    int shift_dx, shift_dy;    /* iterations by (dx, dy) cells; 0: fixed field  */
} orc_loop_opts;

/* Offset of the moving θ field at global iteration T: move_substrate!
 * (scripts/Moving_wettability_structs.jl:139-152) circshifts the field by
 * (dx, dy) at the end of every tmove-th iteration, so iteration T sees it
 * moved k = (T - 1) / tmove times: field(i, j) = θ(i - k dx, j - k dy). */
static void field_shift(const orc_loop_opts *o, long T, int Lx, int Ly, int *sx, int *sy) {
    *sx = 0;
    *sy = 0;
    if (o->shift_tmove <= 0 || T < 1) return;
    const long k = (T - 1) / o->shift_tmove;
    *sx = (int)((k % Lx) * o->shift_dx % Lx);
    *sy = (int)((k % Ly) * o->shift_dy % Ly);
}

/* ------------------------------------------------------------------ */
/* thermal! (src/forcing.jl:297-320): per cell and component a standard  */
/* normal times sqrt(2 kbt mu 6 h / (2h^2 + 6 h delta + 3 delta^2)).     */
/* Julia's randn! stream cannot be reproduced, so the normals come from  */
/* a counter-based generator shared with the GPU: Philox-4x32-10 (Salmon, */
/* Moraes, Dror, Shaw, SC'11) keyed by the seed, counter (cell, t), then  */
/* Box-Muller.  The reference pins only mean 0 and variance 2 kbt/11 at   */
/* h = 1 (test/forcing.jl:141-164).                                       */
/* ------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t x0 = ctr_in[0], x1 = ctr_in[1], x2 = ctr_in[2], x3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
        const uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0, y1 = (uint32_t)p1;
        const uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1, y3 = (uint32_t)p0;
        x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    }
    out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

/* Two standard normals for cell k at time_loop iteration t. */
void orc_thermal_normals(uint64_t seed, uint64_t k, int64_t t, double *zx, double *zy) {
    const uint32_t ctr[4] = {(uint32_t)k, (uint32_t)(uint64_t)t, (uint32_t)((uint64_t)t >> 32),
                             (uint32_t)(k >> 32)};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t w[4];
    orc_philox4x32_10(ctr, key, w);
    const double u1 = (double)((((uint64_t)w[0] << 32) | w[1]) >> 11) * 0x1p-53 + 0x1p-54;
    const double u2 = (double)((((uint64_t)w[2] << 32) | w[3]) >> 11) * 0x1p-53;
    const double r = sqrt(-2.0 * log(u1));
    *zx = r * cos(6.283185307179586 * u2);
    *zy = r * sin(6.283185307179586 * u2);
}

/* thermal!(fx, fy, h, kbt, mu, delta) with the noise of iteration t. */
void orc_thermal(double *fx, double *fy, const double *h, size_t N, double kbt, double mu,
                 double delta, uint64_t seed, int64_t t) {
    for (size_t k = 0; k < N; ++k) {
        double zx, zy;
        orc_thermal_normals(seed, k, t, &zx, &zy);
        const double s = sqrt((((2.0 * kbt) * mu) * 6.0) * h[k] /
                              (((2.0 * h[k]) * h[k] + (6.0 * h[k]) * delta) + (3.0 * delta) * delta));
        fx[k] = zx * s;
        fy[k] = zy * s;
    }
}

/* Per-iteration outputs (each may be NULL): mass (only where t % tdump == 0,
 * NaN elsewhere), Δh, wetted count.  Index t-1 for loop iteration t. */
typedef struct {
    double *mass;
    double *dh;
    int64_t *wet;
} orc_loop_out;

/* time_loop(sys, state[, θ | Δh | f, measure]) -- literal
 * (src/simulate.jl:6-96): each op is one pass over the lattice. */
void orc_time_loop(orc_state *s, const orc_params *P, int Tmax, const orc_loop_opts *o,
                   orc_loop_out *out) {
    int Lx = s->Lx, Ly = s->Ly;
    size_t N = (size_t)Lx * Ly;
    double *moved = (o->theta_field && o->shift_tmove > 0) ? malloc(N * sizeof(double)) : NULL;
    for (int t = 1; t <= Tmax; ++t) {
        const double *theta_field = o->theta_field;
        if (moved) {  /* the field as move_substrate! has left it */
            int sx, sy;
            field_shift(o, o->t_offset + t, Lx, Ly, &sx, &sy);
            orc_circshift(moved, o->theta_field, Lx, Ly, sx, sy);
            theta_field = moved;
        }
        if (out && out->mass) out->mass[t - 1] = (P->tdump > 0 && t % P->tdump == 0)
                                                     ? orc_sum(s->height, N)
                                                     : NAN;
        if (o->record_dh && out && out->dh) out->dh[t - 1] = orc_dh(s->height, N);
        orc_filmpressure(s->pressure, s->height, s->dgrad, Lx, Ly, P->gamma, theta_field,
                         o->theta, P->n, P->m, P->hmin, P->hcrit);
        orc_hgradp(s->hgx, s->hgy, s->height, s->pressure, s->dgrad, Lx, Ly);
        orc_slippage(s->slipx, s->slipy, s->height, s->velx, s->vely, N, P->delta, P->mu);
        orc_force_sum(s->Fx, s->Fy, s->hgx, s->hgy, s->slipx, s->slipy, N);
        if (P->kbt > 0.0) {  /* Fx .= -h∇px .- slipx .- kbtx (scripts/Rivulet_stability.jl:123) */
            for (size_t k = 0; k < N; ++k) {
                double zx, zy;
                orc_thermal_normals(o->thermal_seed, k, o->t_offset + t, &zx, &zy);
                const double hk = s->height[k];
                const double sg = sqrt((((2.0 * P->kbt) * P->mu) * 6.0) * hk /
                                       (((2.0 * hk) * hk + (6.0 * hk) * P->delta) +
                                        (3.0 * P->delta) * P->delta));
                s->Fx[k] = s->Fx[k] - zx * sg;
                s->Fy[k] = s->Fy[k] - zy * sg;
            }
        }
        if (o->callback == 1) {
            if (out && out->wet) out->wet[t - 1] = orc_wetted(s->height, N, o->hthresh);
        } else if (o->callback == 2) {
            long ti = o->incl_loop_time ? (long)t : o->incl_t;
            orc_inclination(s->Fx, s->Fy, s->height, N, o->incl_ax, o->incl_ay, ti,
                            o->incl_tstart, o->incl_tsmooth);
        }
        orc_equilibrium(s->feq, s->height, s->velx, s->vely, s->vsq, N, P->g);
        orc_bgk_stream(s->fout, s->feq, s->ftemp, s->Fx, s->Fy, Lx, Ly, P->tau);
        orc_moments(s->height, s->velx, s->vely, s->fout, N);
    }
    free(moved);
}

/* ------------------------------------------------------------------ */
/* FUSED restatement (OpenMP).  State: post-collision populations fpost */
/* (9N) such that the reference's fout == ftemp == pull(fpost); h/ux/uy */
/* fields are the source of the first step when `fresh` is set (the    */
/* state right after Sys()/height assignment, src/simulate.jl:384-397). */
/* ------------------------------------------------------------------ */
static inline void pull_cell(const double *fp, size_t N, int i, int j, int Lx, int Ly,
                             double ft[9]) {
    for (int q = 0; q < 9; ++q) {
        int si = i - CX[q], sj = j - CY[q];
        if (si < 0) si += Lx; else if (si >= Lx) si -= Lx;
        if (sj < 0) sj += Ly; else if (sj >= Ly) sj -= Ly;
        ft[q] = fp[q * N + IDX(si, sj, Lx)];
    }
}

static inline void nb9(const double *a, int i, int j, int Lx, int Ly, double v[9]) {
    /* v: ip, jp, im, jm, ipjp, imjp, imjm, ipjm of `a` at (i,j), i.e. the
     * values circshift! puts at (i,j): a[i-1,j], a[i,j-1], a[i+1,j], ... */
    int im1 = i == 0 ? Lx - 1 : i - 1, ip1 = i == Lx - 1 ? 0 : i + 1;
    int jm1 = j == 0 ? Ly - 1 : j - 1, jp1 = j == Ly - 1 ? 0 : j + 1;
    v[0] = a[IDX(im1, j, Lx)];
    v[1] = a[IDX(i, jm1, Lx)];
    v[2] = a[IDX(ip1, j, Lx)];
    v[3] = a[IDX(i, jp1, Lx)];
    v[4] = a[IDX(im1, jm1, Lx)];
    v[5] = a[IDX(ip1, jm1, Lx)];
    v[6] = a[IDX(ip1, jp1, Lx)];
    v[7] = a[IDX(im1, jp1, Lx)];
}

/* Runs `nsteps` iterations of time_loop on (fpost, h, ux, uy).  fpost_tmp is
 * scratch of the same size.  On return fpost holds the latest populations
 * and h/ux/uy their moments (what the reference's state holds).  kappa and
 * press are N-sized scratch.  nthreads <= 0 uses the OpenMP default. */
int orc_fused_run(const orc_params *P, double *fpost, double *fpost_tmp, double *h, double *ux,
                  double *uy, double *press, double *kappa_field, int fresh, int nsteps,
                  const orc_loop_opts *o, orc_loop_out *out, int nthreads) {
    const int Lx = P->Lx, Ly = P->Ly;
    const size_t N = (size_t)Lx * Ly;
    const double omeg = 1.0 - 1.0 / P->tau, invtau = 1.0 / P->tau;
    const double kap_s = orc_kappa(o->theta, P->n, P->m, P->hmin);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (o->theta_field) {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < N; ++k) kappa_field[k] = orc_kappa(o->theta_field[k], P->n, P->m, P->hmin);
    }
    for (int t = 1; t <= nsteps; ++t) {
        /* pass 1: moments of the pulled populations (skipped on a fresh state) */
        if (!fresh) {
#pragma omp parallel for schedule(static)
            for (int j = 0; j < Ly; ++j)
                for (int i = 0; i < Lx; ++i) {
                    double ft[9];
                    pull_cell(fpost, N, i, j, Lx, Ly, ft);
                    size_t k = IDX(i, j, Lx);
                    moments_cell(ft, &h[k], &ux[k], &uy[k]);
                }
        }
        fresh = 0;
        if (out && out->mass) out->mass[t - 1] = (P->tdump > 0 && t % P->tdump == 0) ? orc_sum(h, N) : NAN;
        if (o->record_dh && out && out->dh) out->dh[t - 1] = orc_dh(h, N);
        if (o->callback == 1 && out && out->wet) out->wet[t - 1] = orc_wetted(h, N, o->hthresh);
        /* pass 2: film pressure */
        int fsx, fsy;
        field_shift(o, o->t_offset + t, Lx, Ly, &fsx, &fsy);
#pragma omp parallel for schedule(static)
        for (int j = 0; j < Ly; ++j)
            for (int i = 0; i < Lx; ++i) {
                size_t k = IDX(i, j, Lx);
                double v[9];
                nb9(h, i, j, Lx, Ly, v);
                double kap = o->theta_field
                                 ? kappa_field[IDX(wrapi(i - fsx, Lx), wrapi(j - fsy, Ly), Lx)]
                                 : kap_s;
                double x = P->hmin / (h[k] + P->hcrit);
                double p = -P->gamma * (kap * (orc_power_broad(x, P->n) - orc_power_broad(x, P->m)));
                double lap = (2.0 / 3.0) * (((v[1] + v[0]) + v[2]) + v[3]) +
                             (1.0 / 6.0) * (((v[4] + v[5]) + v[6]) + v[7]) - (10.0 / 3.0) * h[k];
                press[k] = p - P->gamma * lap;
            }
        /* pass 3: forces, equilibrium, collision; store post-collision */
        const double sfac = o->callback == 2
                                ? orc_incl_factor(o->incl_loop_time ? (long)t : o->incl_t,
                                                  o->incl_tstart, o->incl_tsmooth)
                                : 0.0;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < Ly; ++j)
            for (int i = 0; i < Lx; ++i) {
                size_t k = IDX(i, j, Lx);
                double v[9], ft[9], fe[9], fo[9];
                nb9(press, i, j, Lx, Ly, v);
                double hk = h[k];
                double hgx = hk * ((-1.0 / 3.0) * (v[0] - v[2]) -
                                   (1.0 / 12.0) * (((v[4] - v[5]) - v[6]) + v[7]));
                double hgy = hk * ((-1.0 / 3.0) * (v[1] - v[3]) -
                                   (1.0 / 12.0) * (((v[4] + v[5]) - v[6]) - v[7]));
                double den = 2.0 * (hk * hk) + (6.0 * P->delta) * hk + 3.0 * (P->delta * P->delta);
                double sx = ((6.0 * P->mu) * hk * ux[k]) / den;
                double sy = ((6.0 * P->mu) * hk * uy[k]) / den;
                double Fx = -hgx - sx, Fy = -hgy - sy;
                if (P->kbt > 0.0) {
                    double zx, zy;
                    orc_thermal_normals(o->thermal_seed, k, o->t_offset + t, &zx, &zy);
                    const double sg = sqrt((((2.0 * P->kbt) * P->mu) * 6.0) * hk /
                                           (((2.0 * hk) * hk + (6.0 * hk) * P->delta) +
                                            (3.0 * P->delta) * P->delta));
                    Fx = Fx - zx * sg;
                    Fy = Fy - zy * sg;
                }
                if (o->callback == 2) {
                    Fx = Fx + (hk * o->incl_ax) * sfac;
                    Fy = Fy + (hk * o->incl_ay) * sfac;
                }
                feq_cell(hk, ux[k], uy[k], P->g, fe);
                pull_cell(fpost, N, i, j, Lx, Ly, ft);
                collide_cell(ft, fe, Fx, Fy, omeg, invtau, fo);
                for (int q = 0; q < 9; ++q) fpost_tmp[q * N + k] = fo[q];
            }
        memcpy(fpost, fpost_tmp, 9 * N * sizeof(double));
    }
    /* final moments: what the reference's state.height/velx/vely hold */
    if (nsteps > 0) {
#pragma omp parallel for schedule(static)
        for (int j = 0; j < Ly; ++j)
            for (int i = 0; i < Lx; ++i) {
                double ft[9];
                pull_cell(fpost, N, i, j, Lx, Ly, ft);
                size_t k = IDX(i, j, Lx);
                moments_cell(ft, &h[k], &ux[k], &uy[k]);
            }
    }
    return 0;
}

/* Streamed populations (the reference's fout) from post-collision ones. */
void orc_pull_all(double *fout, const double *fpost, int Lx, int Ly) {
    size_t N = (size_t)Lx * Ly;
    for (int j = 0; j < Ly; ++j)
        for (int i = 0; i < Lx; ++i) {
            double ft[9];
            pull_cell(fpost, N, i, j, Lx, Ly, ft);
            for (int q = 0; q < 9; ++q) fout[q * N + IDX(i, j, Lx)] = ft[q];
        }
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ================================================================== */
/* One dimension, D1Q3 (literal; each op one pass over the lattice).   */
/* ================================================================== */
static inline int wrap1(int i, int L) { return i < 0 ? i + L : (i >= L ? i - L : i); }

/* filmpressure!(state::LBM_state_1D, sys; θ, γ) (src/pressure.jl:231-256,
 * 285-315 with a γ field).  theta_field / gamma_field may be NULL. */
void orc1_filmpressure(double *p, const double *h, int L, double gamma, const double *gamma_field,
                       const double *theta_field, double theta, int n, int m, double hmin,
                       double hcrit) {
    for (int i = 0; i < L; ++i) {
        const double th = theta_field ? theta_field[i] : theta;
        const double g = gamma_field ? gamma_field[i] : gamma;
        const double kap = (((1.0 - orc_cospi(th)) * (n - 1)) * (m - 1)) / ((n - m) * hmin);
        const double x = hmin / (h[i] + hcrit);
        p[i] = -g * (kap * (orc_power_broad(x, n) - orc_power_broad(x, m)));
    }
    for (int i = 0; i < L; ++i) {
        const double g = gamma_field ? gamma_field[i] : gamma;
        const double hip = h[wrap1(i - 1, L)], him = h[wrap1(i + 1, L)];
        p[i] = p[i] - g * ((hip - 2.0 * h[i]) + him);
    }
}

/* h∇p!(state::LBM_state_1D) (src/forcing.jl:189-198). */
void orc1_hgradp(double *hgp, const double *h, const double *p, int L) {
    for (int i = 0; i < L; ++i)
        hgp[i] = (h[i] * -0.5) * (p[wrap1(i - 1, L)] - p[wrap1(i + 1, L)]);
}

/* slippage!(slip, height, vel, δ, μ) (src/forcing.jl:68-71). */
void orc1_slippage(double *slip, const double *h, const double *u, int L, double delta,
                   double mu) {
    for (int i = 0; i < L; ++i)
        slip[i] = ((6.0 * mu) * h[i] * u[i]) /
                  ((2.0 * (h[i] * h[i]) + (6.0 * delta) * h[i]) + 3.0 * (delta * delta));
}

/* ∇γ!(state) (src/forcing.jl:423-432). */
void orc1_gradgamma(double *dg, const double *gam, int L) {
    for (int i = 0; i < L; ++i)
        dg[i] = (-3.0 / 2.0) * ((gam[wrap1(i - 1, L)] - gam[wrap1(i + 1, L)]) / 2.0);
}

/* equilibrium!(feq, height, velocity, gravity) (src/equilibrium.jl:169-181);
 * feq is L x 3 column-major. */
void orc1_equilibrium(double *feq, const double *h, const double *u, int L, double g) {
    for (int i = 0; i < L; ++i) {
        const double uu = u[i] * u[i];
        feq[i] = h[i] * ((1.0 - (0.5 * g) * h[i]) - uu);
        feq[L + i] = h[i] * (((0.25 * g) * h[i] + 0.5 * u[i]) + 0.5 * uu);
        feq[2 * L + i] = h[i] * (((0.25 * g) * h[i] - 0.5 * u[i]) + 0.5 * uu);
    }
}

/* BGKandStream!(fout, feq, ftemp, F, τ) (src/collide.jl:179-201). */
void orc1_bgk_stream(double *fout, const double *feq, double *ftemp, const double *F, int L,
                     double tau) {
    const double omeg = 1.0 - 1.0 / tau, it = 1.0 / tau;
    double *fo = malloc(3 * (size_t)L * sizeof(double));
    for (int i = 0; i < L; ++i) {
        fo[i] = omeg * ftemp[i] + it * feq[i];
        fo[L + i] = omeg * ftemp[L + i] + it * feq[L + i] + 0.5 * F[i];
        fo[2 * L + i] = omeg * ftemp[2 * L + i] + it * feq[2 * L + i] - 0.5 * F[i];
    }
    for (int i = 0; i < L; ++i) {
        ftemp[i] = fo[i];
        ftemp[L + i] = fo[L + wrap1(i - 1, L)];
        ftemp[2 * L + i] = fo[2 * L + wrap1(i + 1, L)];
    }
    memcpy(fout, ftemp, 3 * (size_t)L * sizeof(double));
    free(fo);
}

/* moments!(height::Vector, vel, fout) (src/moments.jl:54-62). */
void orc1_moments(double *h, double *u, const double *fout, int L) {
    for (int i = 0; i < L; ++i) {
        h[i] = (fout[i] + fout[L + i]) + fout[2 * L + i];
        u[i] = (fout[L + i] - fout[2 * L + i]) / h[i];
    }
}

/* time_loop(sys::SysConst_1D, state[, θ | Δh | wetted!, area])
 * (src/simulate.jl:98-179), and
 * run_gamma's loop (src/simulate.jl:518-556) when gamma_field is given: the
 * pressure uses the γ field and F .= -h∇p .- slip .- ∇γ.  State arrays:
 * fout, ftemp (L x 3), h, u (L).  dh (may be NULL): max - min of h at the
 * start of each iteration. */
void orc1_time_loop(double *fout, double *ftemp, double *h, double *u, const orc_params *P,
                    int Tmax, const double *theta_field, const double *gamma_field,
                    double *dh, int64_t *wet) {
    const int L = P->Lx;
    double *p = malloc((size_t)L * sizeof(double)), *hgp = malloc((size_t)L * sizeof(double));
    double *slip = malloc((size_t)L * sizeof(double)), *F = malloc((size_t)L * sizeof(double));
    double *feq = malloc(3 * (size_t)L * sizeof(double)), *dg = NULL;
    if (gamma_field) {
        dg = malloc((size_t)L * sizeof(double));
        orc1_gradgamma(dg, gamma_field, L);
    }
    for (int t = 1; t <= Tmax; ++t) {
        if (dh) dh[t - 1] = orc_dh(h, (size_t)L);
        orc1_filmpressure(p, h, L, P->gamma, gamma_field, theta_field, P->theta, P->n, P->m,
                          P->hmin, P->hcrit);
        orc1_hgradp(hgp, h, p, L);
        orc1_slippage(slip, h, u, L, P->delta, P->mu);
        for (int i = 0; i < L; ++i) F[i] = dg ? (-hgp[i] - slip[i]) - dg[i] : -hgp[i] - slip[i];
        if (wet) wet[t - 1] = orc_wetted(h, (size_t)L, 0.055);  /* f(measure, state) */
        orc1_equilibrium(feq, h, u, L, P->g);
        orc1_bgk_stream(fout, feq, ftemp, F, L, P->tau);
        orc1_moments(h, u, fout, L);
    }
    free(p); free(hgp); free(slip); free(F); free(feq); free(dg);
}

/* two_droplets(sys; r₁, r₂, θ₁, θ₂, center) (src/initialvalues.jl:277-323). */
void orc1_two_droplets(double *h, int L, double r1, double r2, double th1, double th2, double c1,
                       double c2) {
    for (int i = 1; i <= L; ++i) {
        const double a = sqrt((i - c1) * (i - c1)), b = sqrt((i - c2) * (i - c2));
        double d1 = a <= r1 ? (cos(asin(a / r1)) - orc_cospi(th1)) * r1 : 0.05;
        double d2 = b <= r2 ? (cos(asin(b / r2)) - orc_cospi(th2)) * r2 : 0.05;
        if (d1 < 0) d1 = 0.05;
        if (d2 < 0) d2 = 0.05;
        double v = d1 + d2 - 0.05;
        h[i - 1] = v < 0 ? 0.05 : v;
    }
}
