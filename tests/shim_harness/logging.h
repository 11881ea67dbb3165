/*
 * logging.h -- stand-in for the reference's src/logging.h (see fd.h here):
 * log_fatal prints and exits, as the reference's does after MPI_Abort;
 * log_infoc prints on rank 0.
 */
#ifndef SHIM_HARNESS_LOGGING_H
#define SHIM_HARNESS_LOGGING_H

#include <stdio.h>
#include <stdlib.h>

#define log_fatal(...)                            \
    do {                                          \
        fprintf(stderr, "FATAL: " __VA_ARGS__);   \
        exit(3);                                  \
    } while (0)
#define log_infoc(RANK, ...)                      \
    do {                                          \
        if ((RANK) == 0)                          \
            fprintf(stdout, __VA_ARGS__);         \
    } while (0)

#endif
