/* A plain C caller of libfdfd_cuda: what a Julia ccall (or any C FFI) sees.
 * Compiles against include/fdfd_cuda.h as C11 and runs without a GPU: version,
 * argument validation of every handle entry point, error strings, and the
 * host-only Ritz-pair solver.  Exit status 0 and "ok" on success. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "fdfd_cuda.h"

static int failures = 0;
#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);  \
            ++failures;                                                   \
        }                                                                 \
    } while (0)

static int create(fdfd_handle** h, int Nx, int Ny, int Npx, double dx, double m, int pol, int prec) {
    return fdfd_create(h, Nx, Ny, Npx, 2, dx, 0.05, 1e-6, m, -18.4, pol, prec);
}

/* |a - b| for complex values stored as {re, im} pairs */
static double cdist(const double* a, const double* b) { return hypot(a[0] - b[0], a[1] - b[1]); }

int main(void) {
    const char* v = fdfd_version();
    CHECK(v != NULL && strncmp(v, "fdfd_cuda", 9) == 0);

    /* fdfd_create validates before it touches the GPU; *h is cleared on failure */
    fdfd_handle* h = (fdfd_handle*)&failures;
    CHECK(create(&h, 2, 16, 2, 0.05, 4.0, FDFD_TM, FDFD_PREC_MIXED) == FDFD_EINVAL);
    CHECK(h == NULL);
    CHECK(create(&h, 20, 16, 11, 0.05, 4.0, FDFD_TM, FDFD_PREC_MIXED) == FDFD_EINVAL);
    CHECK(create(&h, 20, 16, 2, 0.0, 4.0, FDFD_TM, FDFD_PREC_MIXED) == FDFD_EINVAL);
    CHECK(create(&h, 20, 16, 2, 0.05, NAN, FDFD_TM, FDFD_PREC_MIXED) == FDFD_EINVAL);
    CHECK(create(&h, 20, 16, 2, 0.05, 4.0, 3, FDFD_PREC_MIXED) == FDFD_EINVAL);
    CHECK(create(&h, 20, 16, 2, 0.05, 4.0, FDFD_TE, 7) == FDFD_EINVAL);
    CHECK(create(&h, 2000, 1100, 2, 0.05, 4.0, FDFD_TM, FDFD_PREC_MIXED) == FDFD_EINVAL); /* b > 1024 */
    CHECK(fdfd_create(NULL, 20, 16, 2, 2, 0.05, 0.05, 1e-6, 4.0, -18.4, FDFD_TM, FDFD_PREC_MIXED) ==
          FDFD_EINVAL);
    CHECK(fdfd_mf_create(&h, 20, 16, 2, 2, 0.05, 0.05, 1e-6, 4.0, -18.4, 17, 1, FDFD_PREC_MIXED) == FDFD_EINVAL);
    CHECK(h == NULL);

    /* every handle entry point rejects a NULL handle */
    double x[2] = {0, 0};
    int npts = 0;
    fdfd_mode mode;
    memset(&mode, 0, sizeof mode);
    fdfd_profile prof;
    CHECK(fdfd_set_refinement(NULL, 1e-10, 10, FDFD_REFINE_GMRES) == FDFD_EINVAL);
    CHECK(fdfd_set_restart(NULL, 20) == FDFD_EINVAL);
    CHECK(fdfd_set_fallback(NULL, 1) == FDFD_EINVAL);
    CHECK(fdfd_set_wait_limit(NULL, 1000) == FDFD_EINVAL);
    CHECK(fdfd_autotune(NULL) == FDFD_EINVAL);
    CHECK(fdfd_set_checkpoint(NULL, 1) == FDFD_EINVAL);
    CHECK(fdfd_checkpoint_info(NULL, NULL, NULL, NULL) == FDFD_EINVAL);
    CHECK(fdfd_get_tuning(NULL, NULL, 0) == -1);
    {
        fdfd_batch* bt = NULL;
        CHECK(fdfd_batch_create(&bt, 0, NULL) == FDFD_EINVAL && bt == NULL);
        CHECK(fdfd_batch_create(NULL, 1, NULL) == FDFD_EINVAL);
        CHECK(fdfd_batch_factor(NULL, x, NULL) == FDFD_EINVAL);
        CHECK(fdfd_batch_stats(NULL, NULL, NULL, NULL) == FDFD_EINVAL);
        fdfd_batch_destroy(NULL);
    }
    CHECK(fdfd_set_device_budget(NULL, 1 << 20) == FDFD_EINVAL);
    CHECK(fdfd_set_eps(NULL, x) == FDFD_EINVAL);
    CHECK(fdfd_factor(NULL, 1.0) == FDFD_EINVAL);
    CHECK(fdfd_solve(NULL, x, 1, x, x, x, NULL) == FDFD_EINVAL);
    CHECK(fdfd_solve_device(NULL, x, 1, x, x, x, NULL) == FDFD_EINVAL);
    CHECK(fdfd_adjoint(NULL, x, x, x, x, x, NULL) == FDFD_EINVAL);
    CHECK(fdfd_adjoint_vjp(NULL, x, x, x, x, NULL) == FDFD_EINVAL);
    CHECK(fdfd_eigfreq(NULL, 1.0, 1, FDFD_WHICH_LM, 1e-10, x, x, x, NULL) == FDFD_EINVAL);
    CHECK(fdfd_get_mode(NULL, 1.0, &mode, 1, x, x, &npts) == FDFD_EINVAL);
    CHECK(fdfd_mode_sources(NULL, 1, x, 1, &mode, x) == FDFD_EINVAL);
    CHECK(fdfd_poynting(NULL, FDFD_TM, x, x, x, x, x) == FDFD_EINVAL);
    CHECK(fdfd_poynting_device(NULL, FDFD_TM, x, x, x, x, x) == FDFD_EINVAL);
    CHECK(fdfd_flux_integral(NULL, FDFD_TM, x, x, FDFD_X, 1, &npts, x) == FDFD_EINVAL);
    CHECK(fdfd_chi3_solve(NULL, x, x, FDFD_CHI3_NEWTON, 1e-12, 50, x, x, x, x, &npts, NULL) == FDFD_EINVAL);
    CHECK(fdfd_mf_set_deps(NULL, x) == FDFD_EINVAL);
    CHECK(fdfd_mf_factor(NULL, 1.0, 0.1) == FDFD_EINVAL);
    CHECK(fdfd_mf_solve(NULL, x, x, x, x, NULL) == FDFD_EINVAL);
    CHECK(fdfd_get_stencil(NULL, x) == FDFD_EINVAL);
    CHECK(fdfd_apply(NULL, x, 1, x) == FDFD_EINVAL);
    CHECK(fdfd_set_profiling(NULL, 1) == FDFD_EINVAL);
    CHECK(fdfd_get_profile(NULL, &prof) == FDFD_EINVAL);
    CHECK(fdfd_residual_noalloc(0, 4, 1, x, x, x, x, x, NULL) == FDFD_EINVAL);
    CHECK(strcmp(fdfd_last_error(NULL), "null handle") == 0);
    fdfd_destroy(NULL);

    /* host-only Ritz-pair solver: an upper-triangular H has its diagonal as
     * eigenvalues, and each returned vector satisfies H v = w v */
    enum { n = 3 };
    const double H[2 * n * n] = {1.0, 0.0,  0.5, -0.25, 2.0, 1.0,
                                 0.0, 0.0,  2.0, 1.0,   -1.0, 0.5,
                                 0.0, 0.0,  0.0, 0.0,   -3.0, 0.5};
    double w[2 * n], V[2 * n * n];
    CHECK(fdfd_debug_hessenberg_eig(n, H, w, V) == FDFD_OK);
    for (int d = 0; d < n; ++d) {
        const double* hd = &H[2 * (d * n + d)];
        double best = 1e300;
        for (int i = 0; i < n; ++i) best = fmin(best, cdist(hd, &w[2 * i]));
        CHECK(best < 1e-12);
    }
    for (int i = 0; i < n; ++i) {
        double nrm = 0, res = 0;
        for (int r = 0; r < n; ++r) {
            double hv[2] = {0, 0};
            for (int c = 0; c < n; ++c) {
                const double* a = &H[2 * (r * n + c)];
                const double* b = &V[2 * (c * n + i)];
                hv[0] += a[0] * b[0] - a[1] * b[1];
                hv[1] += a[0] * b[1] + a[1] * b[0];
            }
            const double* vr = &V[2 * (r * n + i)];
            const double wv[2] = {w[2 * i] * vr[0] - w[2 * i + 1] * vr[1], w[2 * i] * vr[1] + w[2 * i + 1] * vr[0]};
            res += pow(cdist(hv, wv), 2);
            nrm += vr[0] * vr[0] + vr[1] * vr[1];
        }
        CHECK(fabs(sqrt(nrm) - 1.0) < 1e-12);
        CHECK(sqrt(res) < 1e-12);
    }

    if (failures) {
        fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    printf("ok\n");
    return 0;
}
