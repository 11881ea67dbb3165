/*
 * Stand-in for calc_envelope() (reference src/calc_envelope.c:8), the only
 * FFTW user in the reference. It is reached only when MODE==FWI and LNORM==8
 * (reference src/saveseis.c:48-49), never in the forward-modelling path the
 * oracle runs, so it aborts if called. Test infrastructure only.
 */
#include <stdio.h>
#include <stdlib.h>

void calc_envelope(float **datatrace, float **envelope, int ntr, int ns)
{
    (void)datatrace; (void)envelope; (void)ntr; (void)ns;
    fprintf(stderr, "calc_envelope: not available in the single-rank oracle build\n");
    abort();
}
