/*
 * Test infrastructure (oracle only; never linked into the product).
 *
 * Kirkland's cfpix class (ImageSimulation/multislice/cfpix.cpp:115-230) calls
 * eight FFTW3 single-precision entry points.  No FFTW3 library exists on this
 * machine, but the reference tree vendors FFTW 2.1.5 (ImageSimulation/fftw-2.1.5).
 * This file maps the eight FFTW3 calls onto the FFTW 2.1.5 n-d API, compiled
 * with FFTW_ENABLE_FLOAT so fftw_real is float.
 *
 * Sign: FFTW 2 and FFTW 3 share the convention FFTW_FORWARD = -1 (exp(-i...)),
 * FFTW_BACKWARD = +1, unscaled in both directions.  Layout: row-major n0 x n1
 * with n1 contiguous in both APIs.  Plans are always FFTW_ESTIMATE so the
 * arithmetic (and thus any golden vector made with it) is deterministic.
 */
#include <stdlib.h>
#include <stdio.h>
#include "fftw.h"

typedef struct {
    fftwnd_plan plan;
    int n0, n1;
} shim_plan;

void *fftwf_malloc(size_t n)
{
    void *p = NULL;
    if (posix_memalign(&p, 64, n ? n : 1) != 0) return NULL;
    return p;
}

void fftwf_free(void *p) { free(p); }

int fftwf_init_threads(void) { return 1; }

void fftwf_plan_with_nthreads(int n) { (void)n; }

void *fftwf_plan_dft_2d(int n0, int n1, void *in, void *out, int sign, unsigned flags)
{
    (void)in; (void)out; (void)flags;
    shim_plan *s = (shim_plan *)malloc(sizeof(shim_plan));
    if (!s) return NULL;
    s->n0 = n0;
    s->n1 = n1;
    s->plan = fftw2d_create_plan(n0, n1, sign < 0 ? FFTW_FORWARD : FFTW_BACKWARD,
                                 FFTW_ESTIMATE | FFTW_IN_PLACE);
    return s;
}

void fftwf_execute_dft(void *plan, void *in, void *out)
{
    shim_plan *s = (shim_plan *)plan;
    if (in != out) {
        fprintf(stderr, "fftw3 shim: only in-place transforms are mapped\n");
        abort();
    }
    fftwnd_one(s->plan, (fftw_complex *)in, NULL);
}

/* The complex-to-real path (cfpix init mode 2) is not used by the multislice
 * loop; the two symbols exist only so the objects link. */
void *fftwf_plan_dft_c2r_2d(int n0, int n1, void *in, void *out, unsigned flags)
{
    (void)n0; (void)n1; (void)in; (void)out; (void)flags;
    return NULL;
}

void fftwf_execute(void *plan)
{
    (void)plan;
    fprintf(stderr, "fftw3 shim: c2r execution is not mapped\n");
    abort();
}
