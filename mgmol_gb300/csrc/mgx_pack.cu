// Function packing for one task: which localized orbitals may share a
// storage column (FunctionsPacking, src/FunctionsPacking.cc:40-160).
//
//  - the domain is cut into subdivx equal sub-boxes along x, and the
//    localization region of an orbital (a sphere of its radius widened by
//    the subdomain margin, periodic) is listed in every sub-box it reaches,
//    with the reference's geometry and rounding
//    (LocalizationRegions::computeSubdivOverlapGids,
//    src/LocalizationRegions.cc:1039-1099, with the one-task subdomain of
//    setupSubdomainGeometry, :935-967);
//  - two orbitals overlap when some sub-box lists both
//    (LocalizationRegions::overlap, :1103-1119);
//  - the overlap graph is coloured either greedily in decreasing-degree
//    order (greedyColor / greedyMC, src/tools/coloring.cc) or by Recursive
//    Largest First (colorRLF), with the reference's visiting order and tie
//    rules, so that the colours are the reference's colours.
// Host code only.
#include <cmath>
#include <algorithm>
#include <cstdint>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx
{
namespace pack
{
/* dense symmetric 0/1 overlap pattern, diagonal set */
struct Graph
{
    int n;
    std::vector<uint8_t> a; // row-major n x n
    bool at(int i, int j) const { return a[(size_t)i * n + j] != 0; }
};

/* degree-ordering sort: a descending, b permuted alongside; the
 * partition-exchange scheme and pivot (middle element) of the reference's
 * quicksortI_h2l, which fixes the order of equal degrees */
void sort_desc(int* a, int* b, int lo, int hi)
{
    int i = lo, j = hi;
    const int x = a[(lo + hi) / 2];
    do
    {
        while (a[i] > x)
            i++;
        while (a[j] < x)
            j--;
        if (i <= j)
        {
            std::swap(a[i], a[j]);
            std::swap(b[i], b[j]);
            i++;
            j--;
        }
    } while (i <= j);
    if (lo < j) sort_desc(a, b, lo, j);
    if (i < hi) sort_desc(a, b, i, hi);
}

/* greedy multicolouring in decreasing-degree order: each vertex takes the
 * smallest colour no coloured neighbour holds (greedyColor / greedyMC) */
int color_greedy(const Graph& g, std::vector<int>& color)
{
    const int n = g.n;
    std::vector<int> deg(n), ord(n);
    for (int i = 0; i < n; i++)
    {
        int d = 0;
        for (int j = 0; j < n; j++)
            d += g.at(i, j) ? 1 : 0;
        deg[i] = d;
        ord[i] = i;
    }
    if (n > 0) sort_desc(deg.data(), ord.data(), 0, n - 1);
    color.assign(n, -1);
    std::vector<char> used(n + 1, 0);
    int ncol = 0;
    for (int t = 0; t < n; t++)
    {
        const int v = ord[t];
        int top     = -1;
        for (int j = 0; j < n; j++)
            if (g.at(v, j) && color[j] >= 0)
            {
                used[color[j]] = 1;
                top            = std::max(top, color[j]);
            }
        int c = 0;
        while (c <= top && used[c])
            c++;
        for (int k = 0; k <= top; k++)
            used[k] = 0;
        color[v] = c;
        ncol     = std::max(ncol, c + 1);
    }
    return ncol;
}

/* Recursive Largest First: each colour class starts from the uncoloured
 * vertex of largest degree among the uncoloured ones, then repeatedly adds
 * the candidate (uncoloured, not adjacent to the class) with the most
 * neighbours among the vertices the class excludes; ties go to the last
 * vertex of largest count in visiting order (colorRLF's multimap) */
int color_rlf(const Graph& g, std::vector<int>& color)
{
    const int n = g.n;
    color.assign(n, -1);
    std::vector<int> unc(n);
    for (int i = 0; i < n; i++)
        unc[i] = i;
    auto erase = [](std::vector<int>& v, int x) {
        std::vector<int> w;
        w.reserve(v.size());
        for (int y : v)
            if (y != x) w.push_back(y);
        v.swap(w);
    };
    int ncol = 0;
    while (!unc.empty())
    {
        // the vertex of largest degree within the uncoloured set
        int v0 = -1, best = -1;
        for (int j : unc)
        {
            int d = 0;
            for (int i : unc)
                d += g.at(i, j) ? 1 : 0;
            if (d > 0 && d >= best)
            {
                best = d;
                v0   = j;
            }
        }
        erase(unc, v0);
        color[v0] = ncol;
        std::vector<int> u, v;
        for (int i : unc)
            (g.at(i, v0) ? u : v).push_back(i);
        while (!v.empty())
        {
            int u0 = -1, bu = -1;
            for (int j : v)
            {
                int d = 0;
                for (int i : u)
                    d += g.at(i, j) ? 1 : 0;
                if (d >= bu)
                {
                    bu = d;
                    u0 = j;
                }
            }
            color[u0] = ncol;
            erase(unc, u0);
            // the candidates adjacent to u0 (u0 itself included) move to u
            std::vector<int> keep;
            keep.reserve(v.size());
            for (int i : v)
            {
                if (g.at(i, u0))
                    u.push_back(i);
                else
                    keep.push_back(i);
            }
            v.swap(keep);
        }
        ncol++;
    }
    return ncol;
}

} // namespace pack
} // namespace mgx

using namespace mgx;

extern "C" {

int mgx_pack_functions(const mgx_grid* grid, int ghosts, int nfunc, const double* centers,
    const float* radii, int subdivx, int rlf, int* colors, int* ncolors)
{
    if (!grid || !ncolors || nfunc < 0 || (nfunc > 0 && (!centers || !radii || !colors)))
        return fail(MGX_BAD_ARG, "pack: NULL argument");
    if (subdivx < 1 || subdivx > grid->n[0]) return fail(MGX_BAD_ARG, "pack: subdivx %d", subdivx);
    if (ghosts < 0) return fail(MGX_BAD_ARG, "pack: ghosts %d", ghosts);
    for (int i = 0; i < 3; i++)
        if (grid->n[i] < 1 || !(grid->ll[i] > 0.))
            return fail(MGX_BAD_ARG, "pack: grid");
    // the subdomain of the only task (setupSubdomainGeometry): the whole
    // domain from the origin, margin ghosts x |h| (+1e-8), lattice of mesh
    // points L - h
    double h[3], div[3];
    for (int i = 0; i < 3; i++)
    {
        h[i]   = grid->ll[i] / grid->n[i];
        div[i] = grid->ll[i] - h[i];
    }
    double delta = std::sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) + 1.e-8;
    delta *= (double)ghosts;
    const double loc_length = grid->ll[0] / subdivx;
    // sub-boxes each orbital reaches (computeSubdivOverlapGids)
    std::vector<std::vector<char>> in(nfunc, std::vector<char>(subdivx, 0));
    for (int f = 0; f < nfunc; f++)
    {
        const float radius = (float)((double)radii[f] + delta);
        for (int iloc = 0; iloc < subdivx; iloc++)
        {
            // sub-box centre; the origin is 0, so the subdomain's lower
            // corner drops out of the reference's expressions
            const double cc[3] = { 0.5 * ((2 * iloc + 1) * loc_length), 0.5 * div[1],
                0.5 * div[2] };
            double t[3] = { centers[3 * f], centers[3 * f + 1], centers[3 * f + 2] };
            for (int i = 0; i < 3; i++)
            {
                while (t[i] >= cc[i] + 0.5 * grid->ll[i])
                    t[i] -= grid->ll[i];
                while (t[i] < cc[i] - 0.5 * grid->ll[i])
                    t[i] += grid->ll[i];
            }
            double p[3] = { t[0], t[1], t[2] };
            if (p[0] < iloc * loc_length) p[0] = iloc * loc_length;
            if (p[1] < 0.) p[1] = 0.;
            if (p[2] < 0.) p[2] = 0.;
            if (p[0] > (iloc + 1) * loc_length - h[0]) p[0] = (iloc + 1) * loc_length - h[0];
            if (p[1] > div[1]) p[1] = div[1];
            if (p[2] > div[2]) p[2] = div[2];
            const double d2 = (p[0] - t[0]) * (p[0] - t[0]) + (p[1] - t[1]) * (p[1] - t[1])
                              + (p[2] - t[2]) * (p[2] - t[2]);
            if (d2 < radius * radius) in[f][iloc] = 1;
        }
    }
    // overlap graph (LocalizationRegions::overlap), diagonal set
    pack::Graph g;
    g.n = nfunc;
    g.a.assign((size_t)nfunc * nfunc, 0);
    for (int i = 0; i < nfunc; i++)
    {
        g.a[(size_t)i * nfunc + i] = 1;
        for (int j = 0; j < i; j++)
        {
            bool o = false;
            for (int k = 0; k < subdivx && !o; k++)
                o = in[i][k] && in[j][k];
            g.a[(size_t)i * nfunc + j] = g.a[(size_t)j * nfunc + i] = o ? 1 : 0;
        }
    }
    std::vector<int> c;
    *ncolors = rlf ? pack::color_rlf(g, c) : pack::color_greedy(g, c);
    for (int f = 0; f < nfunc; f++)
        colors[f] = c[f];
    return MGX_OK;
}

} // extern "C"
