/*
 * Force-included ahead of every reference source file when the reference is
 * built as a CPU oracle.  The reference reads fields of malloc'ed structs that
 * it never initialises on a single rank (G.smpi[lev].nshareip, Mesh.c:46 and
 * Connection.c:34-57; G.heat[lev].neq_lr, Mesh.c:315); zero-filled allocation
 * gives them the value a fresh heap happens to give, deterministically.
 */
#include <stdlib.h>
#define malloc(n) calloc(1, (n))
