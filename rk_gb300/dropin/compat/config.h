/*
 * Stand-in for the reference's include/config.h when D.c is built outside the
 * reference tree (the GPU host has no copy of it).  Same macro names and
 * defaults (config.h:30-121); override them with -D as the reference's
 * Makefile DEFINES do.
 */
#ifndef RKCU_COMPAT_CONFIG_H_
#define RKCU_COMPAT_CONFIG_H_

#ifndef BRUSS_GRID_SIZE
#define BRUSS_GRID_SIZE 250
#endif
#ifndef BRUSS_ALPHA
#define BRUSS_ALPHA 2E-3
#endif
#ifndef LV_COUNT
#define LV_COUNT 10000
#endif
#ifndef T_START
#define T_START 0.0
#endif
#ifndef T_END
#define T_END 0.1
#endif
#ifndef TOL
#define TOL 1E-9
#endif
#ifndef STEP_LIMIT
#define STEP_LIMIT 200
#endif
#ifndef METHOD
#define METHOD DOPRI54
#endif
/* lock type and padding of the reference's pthreads runtime (config.h:100-121);
   only printed here, as the reference's main does, for log2tab */
#define MUTEX 0
#define SPINLOCK 1
#ifndef LOCKTYPE
#define LOCKTYPE MUTEX
#endif
#ifndef PAD_SIZE
#define PAD_SIZE 128
#endif

#endif
