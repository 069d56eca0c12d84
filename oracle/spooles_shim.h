/* Stand-in declarations for the SPOOLES 2.2 ordering library.
 *
 * Test infrastructure only: used by oracle/build_ref.sh to compile the
 * unmodified reference solver (sdpa_gmp) into oracle/_ref/.  The SPOOLES
 * tarball is not shipped with the reference (external/spooles has only its
 * patches), and the reference only calls SPOOLES from
 * sdpa_chordal.cpp:ordering_bMat when m > 100 AND nBlock > 5
 * (sdpa_chordal.cpp:349-352), i.e. for the sparse-Schur branch.  Every
 * problem this project runs the oracle on has nBlock <= 5, so the dense
 * branch is taken and none of these functions is ever reached; each stub
 * aborts loudly if it is.
 *
 * The seven SPOOLES header names the reference includes
 * (sdpa_chordal.h:37-43) are created by build_ref.sh as one-line files that
 * include this header.
 */
#ifndef SDPG_SPOOLES_SHIM_H
#define SDPG_SPOOLES_SHIM_H
#include <stdio.h>
#include <time.h>

#ifndef CLK_TCK
#define CLK_TCK CLOCKS_PER_SEC
#endif

typedef struct _IV IV;
typedef struct _IVL IVL;
typedef struct _Graph Graph;
typedef struct _ETree ETree;
typedef struct _InpMtx InpMtx;

#define IVL_CHUNKED 1

IVL *IVL_new(void);
void IVL_init1(IVL *ivl, int type, int maxnlist);
void IVL_setList(IVL *ivl, int ilist, int isize, int ivec[]);
int IVL_tsize(IVL *ivl);
int IVL_nlist(IVL *ivl);
void IVL_listAndSize(IVL *ivl, int ilist, int *psize, int **pivec);
int IVL_writeForHumanEye(IVL *ivl, FILE *fp);
void IVL_free(IVL *ivl);
void IV_free(IV *iv);
int *IV_entries(IV *iv);
int IV_size(IV *iv);
Graph *Graph_new(void);
void Graph_init2(Graph *g, int type, int nvtx, int nvbnd, int nedges, int totvewght, int totewght,
                 IVL *adjIVL, IV *vwghtsIV, IVL *ewghtIVL);
void Graph_free(Graph *g);
IV *ETree_newToOldVtxPerm(ETree *etree);
void ETree_free(ETree *etree);
IVL *SymbFac_initFromGraph(ETree *etree, Graph *graph);
ETree *orderViaMMD(Graph *graph, int seed, int msglvl, FILE *msgFile);
ETree *orderViaND(Graph *graph, int maxdomainsize, int seed, int msglvl, FILE *msgFile);
ETree *orderViaMS(Graph *graph, int maxdomainsize, int seed, int msglvl, FILE *msgFile);
ETree *orderViaBestOfNDandMS(Graph *graph, int maxdomainsize, int maxzeros, int maxsize, int seed,
                             int msglvl, FILE *msgFile);

#endif
