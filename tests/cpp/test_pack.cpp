// FunctionsPacking through the C++ adaptor, host only: reads a grid, its
// ghost width, the sub-boxes, the colouring and the regions from stdin and
// prints the number of colours, then each gid's colour.
#include <cstdio>
#include <vector>

#include "mgmol_adaptor.h"

using namespace mgx;

int main()
{
    int n[3], ghosts, subdivx, rlf, nfunc;
    double ll[3];
    if (std::scanf("%d %d %d %lf %lf %lf %d %d %d %d", &n[0], &n[1], &n[2], &ll[0], &ll[1],
            &ll[2], &ghosts, &subdivx, &rlf, &nfunc)
        != 10)
        return 2;
    std::vector<double> c(3 * (size_t)nfunc);
    std::vector<float> r(nfunc);
    for (int f = 0; f < nfunc; f++)
        if (std::scanf("%lf %lf %lf %f", &c[3 * f], &c[3 * f + 1], &c[3 * f + 2], &r[f]) != 4)
            return 2;
    const double origin[3] = { 0., 0., 0. };
    const unsigned pts[3]  = { (unsigned)n[0], (unsigned)n[1], (unsigned)n[2] };
    const pb::Grid g(origin, ll, pts, (short)ghosts);
    FunctionsPacking p(g, c.data(), r.data(), nfunc, subdivx, rlf != 0);
    std::printf("%d\n", (int)p.getNumColors());
    for (int f = 0; f < p.getGlobalSize(); f++)
        std::printf("%d\n", (int)p.getColor(f));
    return 0;
}
