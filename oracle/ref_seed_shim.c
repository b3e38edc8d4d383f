/*
 * Seed override for the reference backend built under oracle/_ref/.
 *
 * The reference master seeds its sampler with srand(getpid())
 * (libcirc/probability.c:182), so two runs never draw the same random
 * stabilizer states.  Linking this object into the reference executable
 * interposes getpid(): when CSIM_REF_SEED is set, the sampler is seeded with
 * that value instead, which makes reference runs reproducible and lets the
 * GPU backend be compared with them sample for sample.  Without the variable
 * the real process id is returned, i.e. the reference behaves as shipped.
 *
 * Test infrastructure only.
 */
#define _GNU_SOURCE
#include <stdlib.h>
#include <sys/syscall.h>
#include <sys/types.h>
#include <unistd.h>

pid_t getpid(void) {
    const char *s = getenv("CSIM_REF_SEED");
    if (s && *s) return (pid_t)strtol(s, NULL, 10);
    return (pid_t)syscall(SYS_getpid);
}
