/* The C ABI used from plain C (C99, -pedantic), as a cgo / JNI / N-API
 * binding uses it: opaque handles, size_t sizes, int statuses and the
 * calling thread's last error.  Only calls that are decided on the host,
 * so it runs without a GPU.  Exit status 0 when every check passes. */
#include <stdio.h>
#include <string.h>

#include "hpxfft_gb300.h"

static int failures = 0;
#define CHECK(cond)                                                        \
    do {                                                                   \
        if (!(cond)) {                                                     \
            fprintf(stderr, "%s:%d: CHECK(%s) failed\n", __FILE__, __LINE__, #cond); \
            ++failures;                                                    \
        }                                                                  \
    } while (0)

int main(void)
{
    hpxfft_plan plan = NULL;
    hpxfft_plan3d plan3 = NULL;
    size_t bytes = 0;
    double value = 0.0;

    CHECK(strcmp(hpxfft_status_string(HPXFFT_OK), "ok") == 0);
    CHECK(hpxfft_plan_flag_valid("estimate") == 1 && hpxfft_plan_flag_valid("Estimate") == 0);

    /* a bad plan flag: HPXFFT_ERR_INVALID_ARG, a message, a null handle */
    CHECK(hpxfft_plan_create(&plan, 4, 6, 1, HPXFFT_PREC_F64, "fastest") == HPXFFT_ERR_INVALID_ARG);
    CHECK(plan == NULL);
    CHECK(strstr(hpxfft_last_error(), "plan flag") != NULL);

    /* sizes decided before any device call */
    CHECK(hpxfft_plan_create(&plan, 4, 5, 1, HPXFFT_PREC_F64, "estimate") == HPXFFT_ERR_UNSUPPORTED_SIZE);
    CHECK(hpxfft_plan_create(&plan, 1024, 36, 1, HPXFFT_PREC_BF16X3, "estimate") == HPXFFT_ERR_UNSUPPORTED_SIZE);
    CHECK(hpxfft_plan_create(&plan, 1000, 6, 1, HPXFFT_PREC_BF16X3, "estimate") == HPXFFT_ERR_UNSUPPORTED_SIZE);
    CHECK(hpxfft_plan_create(&plan, 0, 6, 1, HPXFFT_PREC_F64, "estimate") == HPXFFT_ERR_INVALID_ARG);
    CHECK(hpxfft_plan_create(NULL, 4, 6, 1, HPXFFT_PREC_F64, "estimate") == HPXFFT_ERR_INVALID_ARG);
    CHECK(hpxfft_plan3d_create(&plan3, 4, 4, 6, 1, HPXFFT_PREC_F64, "fastest") == HPXFFT_ERR_INVALID_ARG);
    CHECK(plan3 == NULL);

    /* null handles are reported, never dereferenced */
    CHECK(hpxfft_plan_destroy(NULL) == HPXFFT_ERR_STATE);
    CHECK(hpxfft_execute_r2c(NULL, NULL) == HPXFFT_ERR_STATE);
    CHECK(hpxfft_plan_buffer_bytes(NULL, &bytes) != HPXFFT_OK);
    CHECK(hpxfft_get_measurement(NULL, "total", &value) != HPXFFT_OK);
    CHECK(hpxfft_plan3d_destroy(NULL) == HPXFFT_ERR_STATE);

    /* the tuned-plan cache is host state */
    CHECK(hpxfft_wisdom_forget() == HPXFFT_OK);
    CHECK(hpxfft_wisdom_import("/nonexistent-dir/wisdom.txt") == HPXFFT_ERR_IO);

    if (failures) {
        fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    printf("all C ABI host checks passed\n");
    return 0;
}
