/* C harness of libmgbf's C-ABI (include/mgbf.h), the way a C or Fortran
 * caller binds it.  Without arguments it runs host-only checks (no GPU
 * needed): namelist parsing, handle creation, derived sizes, error codes.
 * With "gpu" it also filters a field in host memory with
 * filtering_procedure(1), prints a checksum and, given a third argument,
 * writes the filtered VALL there as raw doubles. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mgbf.h"

#define CHECK(x)                                                                 \
    do {                                                                         \
        int rc_ = (x);                                                           \
        if (rc_ != MGBF_OK) {                                                    \
            fprintf(stderr, "%s -> %d (%s): %s\n", #x, rc_, mgbf_strerror(rc_), \
                    mgbf_last_error());                                          \
            return 1;                                                            \
        }                                                                        \
    } while (0)

int main(int argc, char** argv) {
    const char* nml = argc > 2 ? argv[2] : "mgbeta.nml";
    mgbf_config cfg;
    CHECK(mgbf_config_init(&cfg));
    char err[256];
    CHECK(mgbf_config_read_namelist(nml, &cfg, err, sizeof err));
    mgbf_handle* h = NULL;
    CHECK(mgbf_create(&cfg, &h));
    mgbf_dims d;
    CHECK(mgbf_get_dims(h, &d));
    printf("im=%d jm=%d km_all=%d gm=%d reach_h=%d reach_z=%d elems=%zu kernel=%d\n", d.im, d.jm, d.km_all, d.gm,
           d.reach_h, d.reach_z, d.field_elems, d.hbeta_kernel);
    /* unknown procedure numbers are a no-op, as in the reference */
    double dummy = 0.0;
    CHECK(mgbf_filtering_procedure(h, 0, &dummy, MGBF_F64, MGBF_MEM_HOST, NULL));
    /* filtering_lin3 (5) is not self-adjoint: its adjoint is refused before any data is touched */
    if (mgbf_filtering_procedure_adjoint(h, 5, &dummy, MGBF_F64, MGBF_MEM_HOST, NULL) != MGBF_ERR_UNSUPPORTED) return 2;
    if (argc > 1 && strcmp(argv[1], "gpu") == 0) {
        double* v = (double*)calloc(d.field_elems, sizeof(double));
        const size_t ni = (size_t)d.im + 2 * d.hx;
        const size_t c = (size_t)d.km_all * ((size_t)(d.im / 2 + d.hx) + ni * (size_t)(d.jm / 2 + d.hy));
        v[c] = 1.0; /* unit impulse at the grid centre, level 1 */
        CHECK(mgbf_filtering_procedure(h, 1, v, MGBF_F64, MGBF_MEM_HOST, NULL));
        double s = 0.0, m = 0.0;
        for (size_t t = 0; t < d.field_elems; ++t) {
            s += v[t];
            if (fabs(v[t]) > m) m = fabs(v[t]);
        }
        printf("impulse response: sum=%.12e max=%.12e\n", s, m);
        if (argc > 3) {
            FILE* f = fopen(argv[3], "wb");
            if (!f || fwrite(v, sizeof(double), d.field_elems, f) != d.field_elems) return 3;
            fclose(f);
        }
        free(v);
    }
    CHECK(mgbf_destroy(h));
    printf("ok\n");
    return 0;
}
