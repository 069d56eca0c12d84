/* Abort stubs for the SPOOLES 2.2 entry points named in spooles_shim.h.
 *
 * Test infrastructure only (linked into oracle/_ref/sdpa_gmp by
 * oracle/build_ref.sh).  The reference reaches SPOOLES only on its
 * sparse-Schur branch (sdpa_chordal.cpp:349-352: m > 100 and nBlock > 5);
 * the oracle is only run on problems with nBlock <= 5, so reaching any of
 * these is a usage error and stops the process with a message.
 */
#include <stdio.h>
#include <stdlib.h>
#include "spooles_shim.h"

static void sdpg_spooles_unreachable(const char *fn) {
    fprintf(stderr, "oracle: SPOOLES function %s reached; the sparse-Schur branch "
                    "(nBlock > 5 and m > 100) is not supported by this oracle build\n", fn);
    abort();
}

#define STUB(ret, name, args) ret name args { sdpg_spooles_unreachable(#name); return (ret)0; }
#define STUBV(name, args) void name args { sdpg_spooles_unreachable(#name); }

STUB(IVL *, IVL_new, (void))
STUBV(IVL_init1, (IVL *ivl, int type, int maxnlist))
STUBV(IVL_setList, (IVL *ivl, int ilist, int isize, int ivec[]))
STUB(int, IVL_tsize, (IVL *ivl))
STUB(int, IVL_nlist, (IVL *ivl))
STUBV(IVL_listAndSize, (IVL *ivl, int ilist, int *psize, int **pivec))
STUB(int, IVL_writeForHumanEye, (IVL *ivl, FILE *fp))
STUBV(IVL_free, (IVL *ivl))
STUBV(IV_free, (IV *iv))
STUB(int *, IV_entries, (IV *iv))
STUB(int, IV_size, (IV *iv))
STUB(Graph *, Graph_new, (void))
STUBV(Graph_init2, (Graph *g, int type, int nvtx, int nvbnd, int nedges, int totvewght,
                    int totewght, IVL *adjIVL, IV *vwghtsIV, IVL *ewghtIVL))
STUBV(Graph_free, (Graph *g))
STUB(IV *, ETree_newToOldVtxPerm, (ETree *etree))
STUBV(ETree_free, (ETree *etree))
STUB(IVL *, SymbFac_initFromGraph, (ETree *etree, Graph *graph))
STUB(ETree *, orderViaMMD, (Graph *graph, int seed, int msglvl, FILE *msgFile))
STUB(ETree *, orderViaND, (Graph *graph, int maxdomainsize, int seed, int msglvl, FILE *msgFile))
STUB(ETree *, orderViaMS, (Graph *graph, int maxdomainsize, int seed, int msglvl, FILE *msgFile))
STUB(ETree *, orderViaBestOfNDandMS, (Graph *graph, int maxdomainsize, int maxzeros, int maxsize,
                                      int seed, int msglvl, FILE *msgFile))
