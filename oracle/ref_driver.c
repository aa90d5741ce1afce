/* ref_driver.c -- a small ctypes-facing driver around the reference engine's own CPU path
 * (engine/cuda/mcg_host.h: mcg_host_load, mcg_ref_points, mcg_ref_tie_mask).  Compiled together
 * with the reference sources by oracle/build.py, only where the reference tree is mounted; it is
 * used to cross-check the oracle restatement (test infrastructure only). */
#include "mcg_host.h"
#include <stdlib.h>

void *ref_open(int version, int dim, const char *preset) {
    McgHost *h = (McgHost *)calloc(1, sizeof *h);
    if (mcg_host_load(h, version, dim, preset)) { free(h); return NULL; }
    return h;
}
void ref_close(void *h) {
    if (!h) return;
    mcg_host_free((McgHost *)h);
    free(h);
}
void ref_points(void *h, const long long *seeds, int ns, const int *pts, int np, unsigned char *out, int *tg) {
    mcg_ref_points((const McgHost *)h, (const i64 *)seeds, ns, (const i32 *)pts, np, out, (i32 *)tg);
}
void ref_tie_mask(void *h, const int tg[6], unsigned long long out[2]) {
    mcg_ref_tie_mask((const McgHost *)h, (const i32 *)tg, (u64 *)out);
}
