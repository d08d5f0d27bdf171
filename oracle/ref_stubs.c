/*
 * ref_stubs.c -- link-time stand-ins for reference symbols that
 * src/libahf/ahf_halos.c and src/libutility/*.c reference but that the
 * unbinding + property stage, the gather and the particle writer never call
 * (logging, grid freeing, MPI termination).  TEST INFRASTRUCTURE ONLY: part of
 * oracle/_ref/libahfref.so.  Each aborts loudly if ever reached.
 */
#include <stdio.h>
#include <stdlib.h>

#define STUB(name) \
  void name(void) { fprintf(stderr, "ref harness: unexpected call to " #name "\n"); abort(); }

STUB(common_terminate)
STUB(io_logging_msg)
STUB(timer_getTime)
