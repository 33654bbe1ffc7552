/*
 * Link check of the drop-in: the reference's own driver sources
 * (photoNs.c initial.c domains.c toptree.c utility.c snapshot.c, compiled
 * with their -fcommon globals and photoNs.c's main renamed) linked against
 * libphotons_fmm.so in place of fmm.c operator.c remotes.c partmesh.c
 * conv.f90.  This main makes no GPU call: it checks that the library's
 * entry points read and write the executable's copies of the reference's
 * globals (the executable's definitions take precedence at load time).
 * Exit status 0 when every check holds; each failure prints a line.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "photoNs.h"
#include "operator.h"

static int fails = 0;
#define CHECK(c, what) do { if (!(c)) { printf("FAIL %s\n", what); fails++; } } while (0)

int main(void)
{
    /* the library's view of a global is the executable's symbol */
    CHECK(dlsym(RTLD_DEFAULT, "cutoffRadius") == (void *)&cutoffRadius, "cutoffRadius resolves to the executable");
    CHECK(dlsym(RTLD_DEFAULT, "part") == (void *)&part, "part resolves to the executable");
    CHECK(dlsym(RTLD_DEFAULT, "walk_m2l_count") == (void *)&walk_m2l_count, "walk_m2l_count resolves to the executable");

    /* acceptance reads the executable's open_angle and cutoffRadius */
    double wi[3] = {1, 1, 1}, wj[3] = {1, 1, 1}, dist[3] = {6, 0, 0};
    open_angle = 0.5;
    cutoffRadius = 4.0;
    CHECK(acceptance(wi, wj, dist) == -1, "acceptance drops a pair beyond the executable's cutoffRadius");
    cutoffRadius = 100.0;
    CHECK(acceptance(wi, wj, dist) == 1, "acceptance accepts it inside the executable's cutoffRadius");
    open_angle = 0.3;
    CHECK(acceptance(wi, wj, dist) == 0, "acceptance opens it with the executable's smaller open_angle");

    /* m2l advances the executable's walk_m2l_count and reads its splitRadius */
    double M[NMULTI], L1[NMULTI], L2[NMULTI];
    for (int i = 0; i < NMULTI; i++) { M[i] = 1.0 / (i + 1); L1[i] = L2[i] = 0.0; }
    walk_m2l_count = 0;
    splitRadius = 1.0;
    m2l(3.0, 1.0, 0.5, M, L1);
    splitRadius = 2.0;
    m2l(3.0, 1.0, 0.5, M, L2);
    CHECK(walk_m2l_count == 2, "m2l counts into the executable's walk_m2l_count");
    CHECK(L1[0] != L2[0], "m2l reads the executable's splitRadius");

    /* p2m reads the executable's part[] and MASSPART */
    Body b[3];
    memset(b, 0, sizeof b);
    for (int i = 0; i < 3; i++) b[i].pos[0] = 1.0 + i;
    part = b;
    MASSPART = 0.25;
    double c[3] = {2.0, 0.0, 0.0}, Mp[NMULTI];
    p2m(0, 3, c, Mp);
    CHECK(fabs(Mp[0] - 0.75) < 1e-15, "p2m sums the executable's MASSPART over its part[]");

    /* fmm_deconstruct releases the executable's toptree (set by the driver) */
    toptree = NULL;
    fmm_deconstruct();
    CHECK(toptree == NULL, "fmm_deconstruct leaves the executable's toptree released");

    printf("%s\n", fails ? "link check failed" : "link check ok");
    return fails ? 1 : 0;
}
