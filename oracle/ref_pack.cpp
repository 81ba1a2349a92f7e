/*
 * ORACLE PINNING DRIVER -- TEST INFRASTRUCTURE ONLY.
 *
 * FunctionsPacking's colouring through the reference MGmol's own
 * src/tools/coloring.cc and SymmetricMatrix (compiled unmodified by
 * oracle/build_ref.sh against the single-task mpi shim): the overlap
 * pattern of n functions in, each function's colour out, numbered in the
 * order of the colour lists as FunctionsPacking::getColors does
 * (src/FunctionsPacking.cc:79-158).  Nothing here is part of the product.
 */
#include <iostream>
#include <list>
#include <vector>

#include "coloring.h"

extern "C" int ref_pack_colors(int n, const unsigned char* overlap, int rlf, int* colors,
    int* ncolors)
{
    std::vector<int> gids(n);
    for (int i = 0; i < n; i++)
        gids[i] = i;
    // FunctionsPacking::setup: the gid-list matrix for RLF, the plain one
    // for the greedy colouring
    SymmetricMatrix<char>* m = rlf ? new SymmetricMatrix<char>(gids, MPI_COMM_WORLD)
                                   : new SymmetricMatrix<char>(n, MPI_COMM_WORLD);
    for (int i = 0; i < n; i++)
    {
        m->setVal(i, i, 1);
        for (int j = 0; j < i; j++)
            m->setVal(i, j, (char)overlap[(size_t)i * n + j]);
    }
    std::list<std::list<int>> cg;
    if (rlf)
        colorRLF(*m, cg, false, std::cout);
    else
        greedyColor(*m, cg, false, std::cout);
    int c = 0;
    for (const auto& l : cg)
    {
        for (int g : l)
            colors[g] = c;
        c++;
    }
    *ncolors = c;
    delete m;
    return 0;
}
