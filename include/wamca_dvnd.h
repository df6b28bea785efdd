/*
 * wamca_dvnd.h -- the reference's extern "C" DVND entry points, exported by
 * libmlpgpu.so with the reference's semantics (including its documented
 * quirks) and implemented on the GB300 engine.
 *
 * Each declaration replaces the reference symbol of the same name:
 *   bestNeighborSimple  source/dvnd.cuh:33, source/dvnd.cu:8-10
 *   bestNeighbor        source/dvnd.cuh:34-36, source/dvnd.cu:12-71
 *   applyMoves          source/dvnd.h:19-20, source/dvnd.cpp:16-145
 *   getNoConflictMoves  source/dvnd.h:22-23, source/dvnd.cpp:155-161
 *   noConflict          source/dvnd.cuh:40, source/dvnd.cu:73-82
 *   segFault            source/dvnd.cpp:230-233
 *
 * Semantics kept from the reference:
 *   - `file` is a TSPLIB EUC_2D instance loaded with costTour = true,
 *     distRound = false (source/dvnd.cpp:163-175).  bestNeighbor loads the
 *     file of its FIRST call and keeps using it for the life of the process
 *     (the function-static problem of source/dvnd.cu:23); applyMoves keeps one
 *     problem per host code 0 the same way (getProblem, dvnd.cpp:163-175).
 *     mlp_legacy_reset() drops both caches (no reference counterpart).
 *   - `solution` holds solutionSize = n + 1 client ids, depot at both ends.
 *   - neighborhood: 0 SWAP, 1 2OPT, 2 OROPT1, 3 OROPT2, 4 OROPT3.
 *   - justCalc: returns the cost of `solution` only.
 *   - *useMoves > 0: up to *useMoves applied moves are written to ids/is/js/
 *     costs, *useMoves becomes the number applied, the resulting tour goes to
 *     solutionResp (if not NULL) and `solution` is left unchanged; with
 *     *useMoves == 0 the resulting tour overwrites `solution`.
 *   - applyMoves applies 2-opt ids (1) as swaps, as the reference does.
 *   - noConflict / getNoConflictMoves reproduce the reference's predicates
 *     and first-conflict marking, typos included.
 * Differences (the reference would crash or misbehave):
 *   - useMoves == NULL is treated as 0 (the reference dereferences it, so
 *     bestNeighborSimple always crashed there).
 *   - Malformed input (bad file, bad tour, bad move) makes the function return
 *     0xFFFFFFFF (bestNeighbor/applyMoves) or -1 (getNoConflictMoves) and
 *     sets mlp_last_error(); the reference threw C++ exceptions through the
 *     C-ABI or exited.
 */
#ifndef WAMCA_DVND_H
#define WAMCA_DVND_H

#include <stdbool.h>
#include <stdint.h>

#include "mlp_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

MLP_API unsigned int bestNeighborSimple(char* file, int* solution, unsigned int solutionSize,
                                        int neighborhood);
MLP_API unsigned int bestNeighbor(char* file, int* solution, unsigned int solutionSize,
                                  int neighborhood, bool justCalc, unsigned int hostCode,
                                  unsigned int* useMoves, unsigned short* ids, unsigned int* is,
                                  unsigned int* js, int* costs, bool useMultipleGpu,
                                  unsigned int deviceCount, int* solutionResp);
MLP_API unsigned int applyMoves(char* file, int* solution, unsigned int solutionSize,
                                unsigned int useMoves, unsigned short* ids, unsigned int* is,
                                unsigned int* js, int* costs);
MLP_API int getNoConflictMoves(unsigned int useMoves, unsigned short* ids, unsigned int* is,
                               unsigned int* js, int* costs, int* selectedMoves, int* impValue,
                               bool maximize, bool melhorParaPior);
MLP_API bool noConflict(unsigned short id1, unsigned int i1, unsigned int j1, unsigned short id2,
                        unsigned int i2, unsigned int j2);
MLP_API void segFault(void);

/* No reference counterpart: drops the problems cached by the calls above. */
MLP_API void mlp_legacy_reset(void);

#ifdef __cplusplus
}
#endif

#endif
