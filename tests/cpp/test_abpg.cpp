// Runs AbpgStep (mgmol_gb300/cpp/abpg_step.h), the C++ host driver of one
// quench iteration, on the block and potential of an input file and writes
// the energies and the final block; tests/test_abpg_cpp_gpu.py writes the
// input and checks the output against the oracle chain and the Python
// schedule.
//
// input:  int32 nx ny nz nfunc dtype(0 FP64, 1 FP32) steps fuse chunk gemm
//         float64 lx ly lz vmin vmax gamma
//         float64 V[npts], then psi[nfunc * npts] of dtype
// output: float64 energies[steps], float64 gamma, then psi of dtype
#include <cstdio>
#include <cstring>
#include <vector>

#include "abpg_step.h"

template <typename T>
int run(FILE* in, FILE* out, const int* hdr, const double* dh)
{
    const unsigned ng[3] = { (unsigned)hdr[0], (unsigned)hdr[1], (unsigned)hdr[2] };
    const int nf = hdr[3], steps = hdr[5];
    const double origin[3] = { 0., 0., 0. };
    const double ll[3]     = { dh[0], dh[1], dh[2] };
    mgx::pb::Grid grid(origin, ll, ng, 0);
    const size_t np = (size_t)ng[0] * ng[1] * ng[2];
    std::vector<double> V(np);
    std::vector<T> psi(np * nf);
    if (fread(V.data(), sizeof(double), np, in) != np) return 2;
    if (fread(psi.data(), sizeof(T), psi.size(), in) != psi.size()) return 2;
    // the potential in the orbital type, as the mixed path keeps it
    std::vector<T> Vt(V.begin(), V.end());
    mgx::DeviceArray<T> dV(np);
    mgx::DeviceArray<T> dpsi(psi.size());
    dV.upload(Vt.data(), np);
    dpsi.upload(psi.data(), psi.size());
    mgx::AbpgOptions o;
    o.fuse_update = hdr[6] != 0;
    o.chunk_funcs = hdr[7];
    o.gemm        = hdr[8];
    o.gamma       = dh[5];
    mgx::AbpgStep<T> step(grid, dV.data(), mgx::dtype_of<T>(), dh[3], dh[4], nf, o);
    std::vector<double> e(steps);
    for (int k = 0; k < steps; k++)
    {
        step.run(dpsi.data());
        e[k] = step.energy();
    }
    dpsi.download(psi.data(), psi.size());
    const double g = step.gamma();
    fwrite(e.data(), sizeof(double), steps, out);
    fwrite(&g, sizeof(double), 1, out);
    fwrite(psi.data(), sizeof(T), psi.size(), out);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc != 3)
    {
        fprintf(stderr, "usage: test_abpg input output\n");
        return 2;
    }
    FILE* in  = fopen(argv[1], "rb");
    FILE* out = fopen(argv[2], "wb");
    if (!in || !out) return 2;
    int hdr[9];
    double dh[6];
    if (fread(hdr, sizeof(int), 9, in) != 9 || fread(dh, sizeof(double), 6, in) != 6) return 2;
    int rc = 1;
    try
    {
        rc = hdr[4] == 0 ? run<double>(in, out, hdr, dh) : run<float>(in, out, hdr, dh);
    }
    catch (const mgx::Error& err)
    {
        fprintf(stderr, "mgx::Error %d: %s\n", err.status, err.what());
        rc = 3;
    }
    fclose(in);
    fclose(out);
    return rc;
}
