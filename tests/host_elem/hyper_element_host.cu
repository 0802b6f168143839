// Host run of hyper_element, the element function of the generic
// HyperElastic kernel (insilico_gb300/csrc/isl_hyper.cu), on inputs written
// by tests/test_host_element_math.py; the stage arrays go back to files.
#include "../../insilico_gb300/csrc/isl_hyper.cu"
#include <cstdio>
#include <cstdlib>
using namespace isl;
template <typename T> std::vector<T> rd(const char* name, size_t n) {
    std::vector<T> v(n);
    if (!n) return v;
    FILE* f = fopen(name, "rb");
    if (!f) { fprintf(stderr, "missing %s\n", name); exit(1); }
    size_t got = fread(v.data(), sizeof(T), n, f);
    fclose(f);
    if (got != n) { fprintf(stderr, "short %s %zu %zu\n", name, got, n); exit(1); }
    return v;
}
template <int SHAPE, int FDEG, int NQ, bool TI>
void run(int E, int nn, int nobj, int mat, int qdeg, int body, int inertia, double massw, int nfw, const double* fw, int nhist) {
    constexpr int D = ET<SHAPE, FDEG>::D, NG = ET<SHAPE, FDEG>::NG, NF = ET<SHAPE, FDEG>::NF;
    HostTab h;
    if (!make_host_tables(SHAPE, FDEG, qdeg, h) || h.nq != NQ) { fprintf(stderr, "tables nq %d\n", h.nq); exit(1); }
    Tab<D, NG, NF, NQ> T;
    fill_tab<SHAPE, FDEG, NQ>(T, h);
    constexpr int NLOC = D * NF, NUP = NLOC * (NLOC + 1) / 2;
    auto X = rd<double>("X.bin", (size_t)nn * D);
    auto conn = rd<int32_t>("conn.bin", (size_t)NG * E);
    auto edof = rd<int32_t>("edof.bin", (size_t)NF * E);
    auto u = rd<double>("u.bin", (size_t)nobj * D);
    auto coef = rd<double>("coef.bin", (size_t)2 * E);
    auto fn = rd<double>("fnodal.bin", body ? (size_t)nn * D : 0);
    auto rho = rd<double>("rho.bin", inertia ? (size_t)E : 0);
    auto hv = rd<double>("hvec.bin", inertia ? (size_t)nobj * D : 0);
    auto hist = rd<double>("hist.bin", (size_t)nhist * nobj * D);
    std::vector<double> SK((size_t)E * NUP), SF((size_t)NLOC * E);
    int flags = 0;
    ElemArgs A;
    memset(&A, 0, sizeof(A));
    A.nelem = E; A.X = X.data(); A.conn = conn.data(); A.edof = edof.data(); A.coef = coef.data(); A.u = u.data();
    A.fnodal = body ? fn.data() : nullptr; A.with_residual = 1; A.general = 1; A.material = mat;
    A.stageK = SK.data(); A.stageF = SF.data(); A.flags = &flags;
    A.rho = inertia ? rho.data() : nullptr; A.mass_w = massw; A.hvec = inertia ? hv.data() : nullptr;
    A.hist = nhist ? hist.data() : nullptr; A.hstride = (int64_t)nobj * D; A.nfw = nfw;
    for (int k = 0; k < nfw; ++k) A.fw[k] = fw[k];
    for (int e = 0; e < E; ++e) hyper_element<SHAPE, FDEG, NQ, double, TI>(A, T, e);
    FILE* f = fopen("SK.bin", "wb"); fwrite(SK.data(), 8, SK.size(), f); fclose(f);
    f = fopen("SF.bin", "wb"); fwrite(SF.data(), 8, SF.size(), f); fclose(f);
    printf("flags %d nup %d\n", flags, NUP);
}
int main(int argc, char** argv) {
    // args: shape E nn nobj deg nq qdeg mat body inertia massw nfw fw0 fw1 nhist
    if (argc != 16) {
        fprintf(stderr, "usage: shape E nn nobj deg nq qdeg mat body inertia massw nfw fw0 fw1 nhist\n");
        return 2;
    }
    int shape = atoi(argv[1]), E = atoi(argv[2]), nn = atoi(argv[3]), nobj = atoi(argv[4]), deg = atoi(argv[5]);
    int nq = atoi(argv[6]), qdeg = atoi(argv[7]), mat = atoi(argv[8]), body = atoi(argv[9]), inertia = atoi(argv[10]);
    double massw = atof(argv[11]);
    int nfw = atoi(argv[12]);
    double fw[2] = {atof(argv[13]), atof(argv[14])};
    int nhist = atoi(argv[15]);
    const bool ti = inertia || nfw > 0;
#define RUN(S, D, Q) if (shape == S && deg == D && nq == Q) { if (ti) run<S, D, Q, true>(E, nn, nobj, mat, qdeg, body, inertia, massw, nfw, fw, nhist); else run<S, D, Q, false>(E, nn, nobj, mat, qdeg, body, inertia, massw, nfw, fw, nhist); return 0; }
    RUN(ISL_QUAD, 1, 4) RUN(ISL_QUAD, 1, 9) RUN(ISL_QUAD, 2, 4) RUN(ISL_QUAD, 2, 9)
    RUN(ISL_TET, 1, 1) RUN(ISL_TET, 1, 4) RUN(ISL_TET, 2, 1) RUN(ISL_TET, 2, 4) RUN(ISL_TET, 2, 11) RUN(ISL_HEX, 1, 27)
    fprintf(stderr, "combo\n");
    return 1;
}
