// Host side of the GB300 assembly + Krylov library: context lifetime, the DOF
// pipeline (DOF-object ids, boundary, constraints, numbering), reference
// element tables, coefficient upload and the extern "C" entry points of
// include/isl_gpu.h.  Device work lives in isl_assembly.cu and isl_solver.cu.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>

#include "isl_internal.h"

using isl::DBuf;

namespace {

// ---------------------------------------------------------------------------
// Reference elements.  Functions are ordered hierarchically (vertices, edge
// interiors, face interiors, cell interior), the order the reference uses for
// Lagrange elements (base/mesh/HierarchicOrder.hpp:161-454).

int sdim(int shape) { return shape == ISL_QUAD ? 2 : 3; }

// 1-D Lagrange basis on [0,1] at equidistant nodes 0, 1/k, .., 1
void lagrange1(int k, double x, double* v, double* d) {
    if (k == 1) {
        v[0] = 1.0 - x; v[1] = x;
        d[0] = -1.0; d[1] = 1.0;
    } else {  // k == 2, nodes 0, 1/2, 1
        v[0] = (1.0 - x) * (1.0 - 2.0 * x); d[0] = 4.0 * x - 3.0;
        v[1] = 4.0 * x * (1.0 - x);         d[1] = 4.0 - 8.0 * x;
        v[2] = x * (2.0 * x - 1.0);         d[2] = 4.0 * x - 1.0;
    }
}

// hierarchic position of every tensor-product node (multi-index i with the
// first coordinate fastest), for degree k in 2-D or 3-D
std::vector<int> cube_positions(int dim, int k) {
    const int n1 = k + 1;
    const int total = dim == 2 ? n1 * n1 : n1 * n1 * n1;
    std::vector<int> pos(total, -1);
    auto lin = [&](int i, int j, int l) { return i + n1 * (j + n1 * l); };
    int c = 0;
    if (dim == 2) {
        const int cx[4] = {0, k, k, 0}, cy[4] = {0, 0, k, k};
        for (int v = 0; v < 4; ++v) pos[lin(cx[v], cy[v], 0)] = c++;
        for (int e = 0; e < 4; ++e) {  // edges v -> v+1, walked from the first vertex
            const int a = e, b = (e + 1) % 4;
            for (int t = 1; t < k; ++t) {
                const int x = cx[a] + (cx[b] - cx[a]) / k * t, y = cy[a] + (cy[b] - cy[a]) / k * t;
                pos[lin(x, y, 0)] = c++;
            }
        }
        for (int j = 1; j < k; ++j)
            for (int i = 1; i < k; ++i) pos[lin(i, j, 0)] = c++;
        return pos;
    }
    const int cx[8] = {0, k, k, 0, 0, k, k, 0}, cy[8] = {0, 0, k, k, 0, 0, k, k}, cz[8] = {0, 0, 0, 0, k, k, k, k};
    for (int v = 0; v < 8; ++v) pos[lin(cx[v], cy[v], cz[v])] = c++;
    const int E[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    for (auto& ed : E)
        for (int t = 1; t < k; ++t) {
            const int a = ed[0], b = ed[1];
            pos[lin(cx[a] + (cx[b] - cx[a]) / k * t, cy[a] + (cy[b] - cy[a]) / k * t, cz[a] + (cz[b] - cz[a]) / k * t)] = c++;
        }
    const int F[6][3] = {{0, 1, 3}, {4, 5, 7}, {0, 1, 4}, {1, 2, 5}, {2, 3, 6}, {3, 0, 7}};  // origin, u-end, v-end
    for (auto& f : F)
        for (int t2 = 1; t2 < k; ++t2)
            for (int t1 = 1; t1 < k; ++t1) {
                const int o = f[0], u = f[1], w = f[2];
                const int x = cx[o] + (cx[u] - cx[o]) / k * t1 + (cx[w] - cx[o]) / k * t2;
                const int y = cy[o] + (cy[u] - cy[o]) / k * t1 + (cy[w] - cy[o]) / k * t2;
                const int z = cz[o] + (cz[u] - cz[o]) / k * t1 + (cz[w] - cz[o]) / k * t2;
                pos[lin(x, y, z)] = c++;
            }
    for (int l = 1; l < k; ++l)
        for (int j = 1; j < k; ++j)
            for (int i = 1; i < k; ++i) pos[lin(i, j, l)] = c++;
    return pos;
}

// values + gradients of the degree-k Lagrange element of a shape at xi
void element_eval(int shape, int k, const double* xi, std::vector<double>& v, std::vector<double>& g, int& nf) {
    if (shape == ISL_TET) {
        const double b1 = xi[0], b2 = xi[1], b3 = xi[2], b0 = 1.0 - b1 - b2 - b3;
        const double db[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        const double b[4] = {b0, b1, b2, b3};
        if (k == 1) {
            nf = 4; v.assign(4, 0); g.assign(12, 0);
            for (int i = 0; i < 4; ++i) { v[i] = b[i]; for (int d = 0; d < 3; ++d) g[i * 3 + d] = db[i][d]; }
            return;
        }
        nf = 10; v.assign(10, 0); g.assign(30, 0);
        for (int i = 0; i < 4; ++i) {
            v[i] = b[i] * (2.0 * b[i] - 1.0);
            for (int d = 0; d < 3; ++d) g[i * 3 + d] = (4.0 * b[i] - 1.0) * db[i][d];
        }
        const int P[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};  // mid-edge functions 4..9
        for (int m = 0; m < 6; ++m) {
            const int i = P[m][0], j = P[m][1];
            v[4 + m] = 4.0 * b[i] * b[j];
            for (int d = 0; d < 3; ++d) g[(4 + m) * 3 + d] = 4.0 * (b[i] * db[j][d] + db[i][d] * b[j]);
        }
        return;
    }
    const int dim = sdim(shape), n1 = k + 1;
    double v1[3][3], d1[3][3];
    for (int d = 0; d < dim; ++d) lagrange1(k, xi[d], v1[d], d1[d]);
    const std::vector<int> pos = cube_positions(dim, k);
    nf = (int)pos.size();
    v.assign(nf, 0); g.assign(nf * dim, 0);
    for (int n = 0; n < nf; ++n) {
        int idx[3] = {n % n1, (n / n1) % n1, n / (n1 * n1)};
        double val = 1.0;
        for (int d = 0; d < dim; ++d) val *= v1[d][idx[d]];
        v[pos[n]] = val;
        for (int a = 0; a < dim; ++a) {
            double gg = 1.0;
            for (int d = 0; d < dim; ++d) gg *= (d == a) ? d1[d][idx[d]] : v1[d][idx[d]];
            g[pos[n] * dim + a] = gg;
        }
    }
}

// Quadrature: Gauss-Legendre on [0,1] with the reference's 15-digit constants
// (base/quad/GaussLegendre.hpp:115-134), tensor products with the first
// coordinate fastest (base/quad/TensorProduct.hpp:123-178), and the
// tetrahedron rules of degree 1 to 5 of base/quad/GaussTetrahedron.hpp.
// surface rules of tetrahedron faces (ISL_TRI: a shape of isl_quadrature_rule only)
constexpr int kTriFace = ISL_TRI;

bool quadrature(int shape, int qdeg, std::vector<double>& w, std::vector<double>& x) {
    w.clear(); x.clear();
    if (shape == kTriFace) {
        // triangle rules of degree 1-5 with the reference's truncated
        // constants and point order (base/quad/GaussTriangle.hpp:97-180):
        // per point the weight, then the two local coordinates
        static const double r1[] = {0.5, 0.333333333333333, 0.333333333333333};
        static const double r2[] = {0.166666666666666, 0.666666666666667, 0.166666666666667,
                                    0.166666666666666, 0.166666666666667, 0.666666666666667,
                                    0.166666666666666, 0.166666666666667, 0.166666666666667};
        static const double r3[] = {-0.28125, 0.333333333333333, 0.333333333333333,
                                    0.260416666666667, 0.6, 0.2,
                                    0.260416666666667, 0.2, 0.6,
                                    0.260416666666667, 0.2, 0.2};
        static const double r4[] = {0.111690794839005, 0.10810301816807, 0.445948490915965,
                                    0.054975871827661, 0.816847572980459, 0.091576213509771,
                                    0.111690794839005, 0.445948490915965, 0.10810301816807,
                                    0.111690794839005, 0.445948490915965, 0.445948490915965,
                                    0.054975871827661, 0.091576213509771, 0.816847572980459,
                                    0.054975871827661, 0.091576213509771, 0.091576213509771};
        static const double r5[] = {0.1125, 0.333333333333333, 0.333333333333333,
                                    0.066197076394253, 0.05971587178977, 0.470142064105115,
                                    0.0629695902724135, 0.797426985353087, 0.101286507323456,
                                    0.066197076394253, 0.470142064105115, 0.05971587178977,
                                    0.066197076394253, 0.470142064105115, 0.470142064105115,
                                    0.0629695902724135, 0.101286507323456, 0.797426985353087,
                                    0.0629695902724135, 0.101286507323456, 0.101286507323456};
        const double* r;
        int np;
        switch (qdeg <= 1 ? 1 : qdeg) {
            case 1: r = r1; np = 1; break;
            case 2: r = r2; np = 3; break;
            case 3: r = r3; np = 4; break;
            case 4: r = r4; np = 6; break;
            case 5: r = r5; np = 7; break;
            default: return false;
        }
        for (int k = 0; k < np; ++k) {
            w.push_back(r[3 * k]);
            x.push_back(r[3 * k + 1]);
            x.push_back(r[3 * k + 2]);
        }
        return true;
    }
    if (shape == ISL_TET) {
        // Keast rules with the reference's truncated constants and point
        // order (base/quad/GaussTetrahedron.hpp:93-175): both decide the last
        // digits of every integral.  Orbits: 'c' the centroid; '4' three
        // coordinates a and one b, in the order (a,a,a) (b,a,a) (a,b,a)
        // (a,a,b); '6' the order (b,b,a) (b,a,a) (a,b,a) (a,a,b) (b,a,b) (a,b,b).
        struct Orbit { char type; double w, a, b; };
        static const Orbit d1[] = {{'c', 0.166666666666666, 0.25, 0.25}};
        static const Orbit d2[] = {{'4', 0.04166666666666666667, 0.13819660112501051518, 0.58541019662496845446}};
        static const Orbit d3[] = {{'c', -0.13333333333333333, 0.25, 0.25}, {'4', 0.075, 0.1666666666666667, 0.5}};
        static const Orbit d4[] = {{'c', -0.01315555555555555556, 0.25, 0.25},
                                   {'4', 0.0076222222222222, 0.071428571428571, 0.785714285714286},
                                   {'6', 0.024888888888889, 0.100596423833201, 0.399403576166799}};
        static const Orbit d5[] = {{'c', 0.030283678097089, 0.25, 0.25},
                                   {'4', 0.006026785714286, 0.333333333333333, 0.0},
                                   {'4', 0.011645249086029, 0.090909090909091, 0.727272727272727},
                                   {'6', 0.010949141561386, 0.066550153573664, 0.433449846426336}};
        const Orbit* rule;
        int norb;
        switch (qdeg <= 1 ? 1 : qdeg) {
            case 1: rule = d1; norb = 1; break;
            case 2: rule = d2; norb = 1; break;
            case 3: rule = d3; norb = 2; break;
            case 4: rule = d4; norb = 3; break;
            case 5: rule = d5; norb = 4; break;
            default: return false;
        }
        for (int o = 0; o < norb; ++o) {
            const double a = rule[o].a, b = rule[o].b;
            const double c4[4][3] = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
            const double c6[6][3] = {{b, b, a}, {b, a, a}, {a, b, a}, {a, a, b}, {b, a, b}, {a, b, b}};
            const int np = rule[o].type == 'c' ? 1 : rule[o].type == '4' ? 4 : 6;
            for (int k = 0; k < np; ++k) {
                const double* pt = rule[o].type == 'c' ? nullptr : rule[o].type == '4' ? c4[k] : c6[k];
                w.push_back(rule[o].w);
                for (int d = 0; d < 3; ++d) x.push_back(pt ? pt[d] : 0.25);
            }
        }
        return true;
    }
    std::vector<double> w1, x1;
    switch ((qdeg + 2) / 2) {
        case 1: w1 = {1.0}; x1 = {0.5}; break;
        case 2: w1 = {0.5, 0.5}; x1 = {0.788675134594813, 0.211324865405187}; break;
        case 3: w1 = {0.277777777777777, 0.444444444444444, 0.277777777777777};
                x1 = {0.887298334620741, 0.5, 0.112701665379259}; break;
        default: return false;
    }
    const int dim = (shape == 0) ? 1 : sdim(shape);
    const int n = (int)w1.size();
    int total = 1;
    for (int d = 0; d < dim; ++d) total *= n;
    w.resize(total); x.resize((size_t)total * dim);
    for (int p = 0; p < total; ++p) {
        int r = p;
        double ww = 1.0;
        for (int d = 0; d < dim; ++d) {
            const int i = r % n; r /= n;
            ww = (d == 0) ? w1[i] : ww * w1[i];
            x[(size_t)p * dim + d] = x1[i];
        }
        w[p] = ww;
    }
    return true;
}

}  // namespace

namespace isl {

bool make_host_tables(int shape, int fedeg, int qdeg, HostTab& t) {
    t = HostTab();
    if (!quadrature(shape, qdeg, t.w, t.xi)) return false;
    t.dim = sdim(shape);
    t.nq = (int)t.w.size();
    std::vector<double> v, g;
    int nf = 0, ng = 0;
    for (int q = 0; q < t.nq; ++q) {
        const double* xi = &t.xi[(size_t)q * t.dim];
        element_eval(shape, fedeg, xi, v, g, nf);
        t.phi.insert(t.phi.end(), v.begin(), v.end());
        t.dphi.insert(t.dphi.end(), g.begin(), g.end());
        element_eval(shape, 1, xi, v, g, ng);
        t.N.insert(t.N.end(), v.begin(), v.end());
        t.dN.insert(t.dN.end(), g.begin(), g.end());
    }
    t.nf = nf;
    t.ng = ng;
    return true;
}

// element face tables (base/mesh/ElementFaces.hpp:282-436)
static const int kQuadEdges[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
static const int kTetFaces[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};
static const int kHexFaces[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};

static void vertex_local_coords(int shape, std::vector<double>& c) {
    if (shape == ISL_QUAD) c = {0, 0, 1, 0, 1, 1, 0, 1};
    else if (shape == ISL_HEX) c = {0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0, 0, 0, 1, 1, 0, 1, 1, 1, 1, 0, 1, 1};
    else c = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
}

bool make_face_tables(int shape, int fedeg, int sqdeg, FaceTab& t) {
    t = FaceTab();
    t.dim = sdim(shape);
    std::vector<double> sw, sx;
    int sshape;
    if (shape == ISL_QUAD) { t.nfaces = 4; t.nfv = 2; sshape = 0; }
    else if (shape == ISL_HEX) { t.nfaces = 6; t.nfv = 4; sshape = ISL_QUAD; }
    else { t.nfaces = 4; t.nfv = 3; sshape = kTriFace; }
    if (!quadrature(sshape, sqdeg, sw, sx)) return false;
    t.nsq = (int)sw.size();
    t.w = sw;
    for (int f = 0; f < t.nfaces; ++f)
        for (int v = 0; v < t.nfv; ++v)
            t.fv.push_back(shape == ISL_QUAD ? kQuadEdges[f][v] : shape == ISL_HEX ? kHexFaces[f][v] : kTetFaces[f][v]);
    std::vector<double> vc;
    vertex_local_coords(shape, vc);
    const int sd = t.dim - 1;
    // surface geometry functions: line [1-e, e], linear triangle [1-a-b, a, b]
    // or hierarchic bilinear quad
    t.dS.assign((size_t)t.nsq * t.nfv * sd, 0.0);
    std::vector<double> sval((size_t)t.nsq * t.nfv);
    for (int q = 0; q < t.nsq; ++q) {
        if (t.nfv == 3) {
            const double a = sx[q * 2], b = sx[q * 2 + 1];
            const double vv[3] = {1 - a - b, a, b}, da[3] = {-1, 1, 0}, db[3] = {-1, 0, 1};
            for (int v = 0; v < 3; ++v) {
                sval[q * 3 + v] = vv[v];
                t.dS[(q * 3 + v) * 2 + 0] = da[v];
                t.dS[(q * 3 + v) * 2 + 1] = db[v];
            }
        } else if (sd == 1) {
            const double e = sx[q];
            sval[q * 2 + 0] = 1 - e; sval[q * 2 + 1] = e;
            t.dS[(q * 2 + 0)] = -1; t.dS[(q * 2 + 1)] = 1;
        } else {
            const double a = sx[q * 2], b = sx[q * 2 + 1];
            const double vv[4] = {(1 - a) * (1 - b), a * (1 - b), a * b, (1 - a) * b};
            const double da[4] = {-(1 - b), (1 - b), b, -b}, db[4] = {-(1 - a), -a, a, (1 - a)};
            for (int v = 0; v < 4; ++v) {
                sval[q * 4 + v] = vv[v];
                t.dS[(q * 4 + v) * 2 + 0] = da[v];
                t.dS[(q * 4 + v) * 2 + 1] = db[v];
            }
        }
    }
    t.S = sval;
    std::vector<double> v, g;
    int nf = 0;
    for (int f = 0; f < t.nfaces; ++f)
        for (int q = 0; q < t.nsq; ++q) {
            double xi[3] = {0, 0, 0};
            for (int k = 0; k < t.nfv; ++k) {
                const int lv = t.fv[f * t.nfv + k];
                for (int d = 0; d < t.dim; ++d) xi[d] += vc[lv * t.dim + d] * sval[q * t.nfv + k];
            }
            element_eval(shape, fedeg, xi, v, g, nf);
            t.phi.insert(t.phi.end(), v.begin(), v.end());
        }
    t.nf = nf;
    return true;
}

}  // namespace isl

// ===========================================================================
// DOF pipeline helpers
namespace {

int num_vertices(int shape) { return shape == ISL_HEX ? 8 : 4; }

// n-face vertex tables of an element (n = 0 vertices, 1 edges, 2 faces, 3 cell)
std::vector<std::vector<int>> nfaces(int shape, int n) {
    static const int tetE[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 1}, {3, 2}};
    static const int hexE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    std::vector<std::vector<int>> t;
    const int nv = num_vertices(shape);
    if (n == 0) { for (int v = 0; v < nv; ++v) t.push_back({v}); return t; }
    if (n == 1) {
        if (shape == ISL_QUAD) for (auto& e : isl::kQuadEdges) t.push_back({e[0], e[1]});
        if (shape == ISL_TET) for (auto& e : tetE) t.push_back({e[0], e[1]});
        if (shape == ISL_HEX) for (auto& e : hexE) t.push_back({e[0], e[1]});
        return t;
    }
    if (n == 2) {
        if (shape == ISL_QUAD) t.push_back({0, 1, 2, 3});
        if (shape == ISL_TET) for (auto& f : isl::kTetFaces) t.push_back({f[0], f[1], f[2]});
        if (shape == ISL_HEX) for (auto& f : isl::kHexFaces) t.push_back({f[0], f[1], f[2], f[3]});
        return t;
    }
    if (n == 3 && shape != ISL_QUAD) {
        std::vector<int> all(nv);
        std::iota(all.begin(), all.end(), 0);
        t.push_back(all);
    }
    return t;
}

// interior DOFs of an n-face of a degree-k Lagrange element
int interior_dofs(int shape, int k, int n) {
    if (n == 0) return 1;
    if (shape == ISL_TET) {
        if (n == 1) return k - 1;
        if (n == 2) return (k - 1) * (k - 2) / 2;
        return (k - 1) * (k - 2) * (k - 3) / 6;
    }
    int r = 1;
    for (int i = 0; i < n; ++i) r *= (k - 1);
    return r;
}

using Key = std::array<int64_t, 4>;

Key face_key(const int64_t* ev, const std::vector<int>& f) {
    Key k = {INT64_MAX, INT64_MAX, INT64_MAX, INT64_MAX};
    for (size_t i = 0; i < f.size(); ++i) k[i] = ev[f[i]];
    std::sort(k.begin(), k.begin() + f.size());
    return k;
}

// Group identical faces: returns, for every (element, face) slot, the slot of
// its first occurrence in element-major order, and the sorted order of keys.
void group_faces(const std::vector<Key>& keys, std::vector<int64_t>& first, std::vector<int64_t>& order) {
    // sort contiguous (key, slot) records: the slot breaks ties, which is the
    // order of a stable sort of the slots by key
    struct Rec {
        Key k;
        int64_t s;
        bool operator<(const Rec& o) const { return k < o.k || (k == o.k && s < o.s); }
    };
    const int64_t n = (int64_t)keys.size();
    std::vector<Rec> rec((size_t)n);
    for (int64_t i = 0; i < n; ++i) rec[i] = {keys[i], i};
    std::sort(rec.begin(), rec.end());
    order.resize(n);
    first.assign(n, -1);
    int64_t i = 0;
    while (i < n) {
        int64_t j = i;
        while (j < n && rec[j].k == rec[i].k) ++j;
        const int64_t f0 = rec[i].s;  // the smallest slot of the group comes first
        for (int64_t k = i; k < j; ++k) {
            order[k] = rec[k].s;
            first[rec[k].s] = f0;
        }
        i = j;
    }
}

}  // namespace

// ===========================================================================
namespace {

// Neumann faces grouped by element for k_neumann; traction per face
// ([n][ncomp]) or, with vertex, per face vertex ([n][nfv][ncomp]).
int neumann_faces(isl_ctx* c, int64_t n, const int64_t* elem, const int* face, const double* traction, bool vertex,
                  int squad_degree) {
    if (!c || !c->fedeg) return ISL_ERR_ARG;
    c->n_neu_elem = 0;
    if (n <= 0) return ISL_OK;
    if (!elem || !face || !traction) return ISL_ERR_ARG;
    const int nfc = c->shape == ISL_HEX ? 6 : 4;
    const int nval = (vertex ? (c->shape == ISL_QUAD ? 2 : c->shape == ISL_TET ? 3 : 4) : 1) * c->ncomp;
    std::vector<int64_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    for (int64_t i = 0; i < n; ++i)
        if (elem[i] < 0 || elem[i] >= c->nelem || face[i] < 0 || face[i] >= nfc) ISL_FAIL(c, ISL_ERR_ARG, "Neumann face out of range");
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return elem[a] < elem[b]; });
    std::vector<int32_t> el, off, fc;
    std::vector<double> tr;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t i = idx[k];
        if (el.empty() || el.back() != elem[i]) { el.push_back((int32_t)elem[i]); off.push_back((int32_t)k); }
        fc.push_back(face[i]);
        for (int d = 0; d < nval; ++d) tr.push_back(traction[i * nval + d]);
    }
    off.push_back((int32_t)n);
    c->n_neu_elem = (int64_t)el.size();
    c->neu_vertex = vertex;
    c->sqdeg = squad_degree;
    ISL_CHECK_CUDA(c, c->dneu_elem.alloc(el.size()));
    ISL_CHECK_CUDA(c, c->dneu_off.alloc(off.size()));
    ISL_CHECK_CUDA(c, c->dneu_face.alloc(fc.size()));
    ISL_CHECK_CUDA(c, c->dneu_trac.alloc(tr.size()));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dneu_elem.p, el.data(), el.size() * 4, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dneu_off.p, off.data(), off.size() * 4, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dneu_face.p, fc.data(), fc.size() * 4, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dneu_trac.p, tr.data(), tr.size() * 8, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

// ---------------------------------------------------------------------------
// Tuning cache.  Key: tuner, element shape, field degree, components,
// kernel, node-blocked, batched, and the size class floor(log2(equations))
// (the rows per launch that decide which variant wins).  File format: one
// "key value" line per entry, appended as entries are found.
namespace {
std::mutex g_tune_mu;
std::map<std::string, int> g_tune;
std::string g_tune_path;
bool g_tune_init = false;

void tune_read_locked(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char key[256];
    int v = 0;
    while (std::fscanf(f, "%255s %d", key, &v) == 2) g_tune[key] = v;
    std::fclose(f);
}

void tune_init_locked() {
    if (g_tune_init) return;
    g_tune_init = true;
    const char* env = std::getenv("ISL_TUNE_CACHE");
    if (env && *env) {
        g_tune_path = env;
        tune_read_locked(g_tune_path);
    }
}

std::string tune_key(const isl_ctx* c, const char* tuner) {
    int cls = 0;
    for (int64_t n = std::max<int64_t>(1, c->neq); n > 1; n >>= 1) ++cls;
    char buf[160];
    std::snprintf(buf, sizeof buf, "%s:s%d:p%d:c%d:k%d:m%d:b%d:i%d:n%d", tuner, c->shape, c->fedeg, c->ncomp, c->kernel,
                  c->material, c->blocked ? 1 : 0, c->ninst > 1 ? 1 : 0, cls);
    return buf;
}
}  // namespace

namespace isl {
bool tune_lookup(const isl_ctx* c, const char* tuner, int* value) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_init_locked();
    auto it = g_tune.find(tune_key(c, tuner));
    if (it == g_tune.end()) return false;
    *value = it->second;
    return true;
}

void tune_store(isl_ctx* c, const char* tuner, int value) {
    c->tune_runs++;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_init_locked();
    const std::string key = tune_key(c, tuner);
    g_tune[key] = value;
    if (!g_tune_path.empty()) {
        if (FILE* f = std::fopen(g_tune_path.c_str(), "a")) {
            std::fprintf(f, "%s %d\n", key.c_str(), value);
            std::fclose(f);
        }
    }
}
}  // namespace isl

extern "C" {

int isl_tune_cache(const char* path) {
    ISL_TRY
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_init = true;
    g_tune.clear();
    g_tune_path = path ? path : "";
    if (!g_tune_path.empty()) tune_read_locked(g_tune_path);
    return ISL_OK;
    ISL_CATCH(nullptr)
}

int isl_ctx_create(isl_ctx** out, int device, void* stream) {
    ISL_TRY
    if (!out) return ISL_ERR_ARG;
    *out = nullptr;
    isl_ctx* c = new isl_ctx();
    c->device = device;
    if (device < 0) {  // host-only context: DOF pipeline without a GPU
        *out = c;
        return ISL_OK;
    }
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete c; return ISL_ERR_CUDA; }
    if (stream) c->stream = (cudaStream_t)stream;
    else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return ISL_ERR_CUDA; }
        c->own_stream = true;
    }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaMallocHost(&c->hscal, sizeof(isl::CGScal)) != cudaSuccess) { delete c; return ISL_ERR_NOMEM; }
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    for (auto& ev : c->mark) cudaEventCreate(&ev);
    if (c->dflags.alloc(4) != cudaSuccess) { delete c; return ISL_ERR_NOMEM; }
    cudaMemsetAsync(c->dflags.p, 0, 4 * sizeof(int), c->stream);
    *out = c;
    return ISL_OK;
    ISL_CATCH(nullptr)
}

int isl_ctx_destroy(isl_ctx* c) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    if (c->device < 0) { delete c; return ISL_OK; }
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& ev : c->ev) if (ev) cudaEventDestroy(ev);
    for (auto& ev : c->mark) if (ev) cudaEventDestroy(ev);
    if (c->hscal) cudaFreeHost(c->hscal);
    cudaStream_t own = c->own_stream ? c->stream : nullptr;
    delete c;  // frees the device buffers (stream-ordered)
    cudaStreamSynchronize(cudaStreamPerThread);
    if (own) cudaStreamDestroy(own);
    return ISL_OK;
    ISL_CATCH(c)
}

const char* isl_last_error(const isl_ctx* c) { return c ? c->err.c_str() : "null context"; }

static int mesh_upload_impl(isl_ctx* c, int shape, int dim, int64_t n_nodes, const double* X, int64_t n_elem,
                            const int64_t* conn, int64_t n_inst, const int64_t* node_off, const int64_t* elem_off);

int isl_mesh_upload(isl_ctx* c, int shape, int dim, int64_t n_nodes, const double* X, int64_t n_elem, const int64_t* conn) {
    ISL_TRY
    const int64_t no[2] = {0, n_nodes}, eo[2] = {0, n_elem};
    return mesh_upload_impl(c, shape, dim, n_nodes, X, n_elem, conn, 1, no, eo);
    ISL_CATCH(c)
}

int isl_batch_mesh_upload(isl_ctx* c, int shape, int dim, int64_t n_inst, const int64_t* node_off, const double* X,
                          const int64_t* elem_off, const int64_t* conn) {
    ISL_TRY
    if (!c || n_inst <= 0 || !node_off || !elem_off) return ISL_ERR_ARG;
    return mesh_upload_impl(c, shape, dim, node_off[n_inst], X, elem_off[n_inst], conn, n_inst, node_off, elem_off);
    ISL_CATCH(c)
}

static int mesh_upload_impl(isl_ctx* c, int shape, int dim, int64_t n_nodes, const double* X, int64_t n_elem,
                            const int64_t* conn, int64_t n_inst, const int64_t* node_off, const int64_t* elem_off) {
    if (!c) return ISL_ERR_ARG;
    if (!(shape == ISL_QUAD || shape == ISL_TET || shape == ISL_HEX)) ISL_FAIL(c, ISL_ERR_ARG, "unsupported shape");
    if (dim != sdim(shape)) ISL_FAIL(c, ISL_ERR_ARG, "dim does not match shape");
    if (n_nodes <= 0 || n_elem <= 0 || !X || !conn) ISL_FAIL(c, ISL_ERR_ARG, "empty mesh");
    if (n_nodes >= INT32_MAX || n_elem >= INT32_MAX) ISL_FAIL(c, ISL_ERR_ARG, "mesh too large for 32-bit ids");
    c->shape = shape; c->dim = dim; c->nnodes = n_nodes; c->nelem = n_elem;
    c->ngeom = num_vertices(shape);
    c->hX.assign(X, X + n_nodes * dim);
    c->hconn.assign(conn, conn + n_elem * c->ngeom);
    if (node_off[0] != 0 || elem_off[0] != 0) ISL_FAIL(c, ISL_ERR_ARG, "instance offsets must start at 0");
    for (int64_t k = 0; k < n_inst; ++k) {
        if (node_off[k + 1] <= node_off[k] || elem_off[k + 1] <= elem_off[k]) ISL_FAIL(c, ISL_ERR_ARG, "empty instance");
        for (int64_t i = elem_off[k] * c->ngeom; i < elem_off[k + 1] * c->ngeom; ++i)
            if (conn[i] < node_off[k] || conn[i] >= node_off[k + 1])
                ISL_FAIL(c, ISL_ERR_ARG, "connectivity out of range (elements must use their own instance's nodes)");
    }
    c->ninst = n_inst;
    c->inst_node_off.assign(node_off, node_off + n_inst + 1);
    c->inst_elem_off.assign(elem_off, elem_off + n_inst + 1);
    c->fedeg = 0; c->numbered = false; c->nnz = 0; c->solved = false; c->mesh_affine = -1; c->mesh_uniform = -1;
    c->bf_valid = false; c->bf_cache.clear();
    if (c->device < 0) return ISL_OK;
    cudaSetDevice(c->device);
    std::vector<int32_t> soa((size_t)n_elem * c->ngeom);
    for (int64_t e = 0; e < n_elem; ++e)
        for (int v = 0; v < c->ngeom; ++v) soa[(size_t)v * n_elem + e] = (int32_t)conn[e * c->ngeom + v];
    ISL_CHECK_CUDA(c, c->dX.alloc(n_nodes * dim));
    ISL_CHECK_CUDA(c, c->dconn.alloc(soa.size()));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dX.p, X, n_nodes * dim * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dconn.p, soa.data(), soa.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
}

// DOF-object ids.  Isoparametric fields copy the node ids
// (base/dof/copyConnectivity.hpp:33-62); otherwise vertices, edges, faces and
// cells are numbered by first visit in element order, shared n-faces copying
// the ids of their first occurrence (base/dof/generateDoFIndicesFromFaces.hpp:169-298).
int isl_field_create(isl_ctx* c, int fe_degree, int ncomp, int64_t* n_dofobj, int* n_fun) {
    ISL_TRY
    if (!c || c->nelem == 0) return ISL_ERR_ARG;
    if (fe_degree < 1 || fe_degree > 3 || ncomp < 1 || ncomp > 3) ISL_FAIL(c, ISL_ERR_ARG, "unsupported field");
    if (c->shape == ISL_TET && fe_degree > 2) ISL_FAIL(c, ISL_ERR_ARG, "tet degree > 2 unsupported");
    c->fedeg = fe_degree; c->ncomp = ncomp;
    const int D = c->dim;
    int nf = 0;
    for (int n = 0; n <= D; ++n) nf += (int)nfaces(c->shape, n).size() * interior_dofs(c->shape, fe_degree, n);
    c->nfun = nf;
    c->nloc = nf * ncomp;
    c->nup = c->nloc * (c->nloc + 1) / 2;
    const int64_t E = c->nelem;
    c->hedof.assign((size_t)E * nf, -1);
    c->inst_dof_off.assign(c->ninst + 1, 0);
    // the shared n-faces of every level, for the device numbering
    std::vector<isl::DeviceLevel> levels;
    int max_nfc = 0;
    if (fe_degree > 1) {
        int begin = 0;
        for (int n = 0; n <= D; ++n) {
            const auto tab = nfaces(c->shape, n);
            isl::DeviceLevel lv;
            lv.nfc = (int)tab.size();
            lv.stride = interior_dofs(c->shape, fe_degree, n);
            lv.begin = begin;
            lv.w = n < D ? (int)(lv.nfc ? tab[0].size() : 0) : 0;
            for (int f = 0; f < lv.nfc && n < D; ++f)
                for (int i = 0; i < lv.w; ++i) lv.v[f][i] = tab[f][i];
            begin += lv.nfc * lv.stride;
            max_nfc = std::max(max_nfc, lv.nfc);
            if (lv.nfc) levels.push_back(lv);
        }
    }
    const bool on_device = fe_degree > 1 && !c->host_setup && isl::device_setup_fits(c, max_nfc);
    if (on_device) {
        cudaSetDevice(c->device);
        const int rc = isl::device_dofobj_numbering(c, levels, nf);
        if (rc != ISL_OK) return rc;
    } else if (fe_degree == 1) {
        int64_t mx = 0;
        for (int64_t i = 0; i < E * nf; ++i) { c->hedof[i] = c->hconn[i]; mx = std::max(mx, c->hconn[i] + 1); }
        c->ndofobj = mx;
        c->inst_dof_off = c->inst_node_off;
        c->inst_dof_off[c->ninst] = mx;
    } else {
        // numbered per instance (each instance exactly as the reference numbers
        // a single mesh), instances concatenated
        int64_t counter = 0;
        for (int64_t k = 0; k < c->ninst; ++k) {
            c->inst_dof_off[k] = counter;
            const int64_t e_lo = c->inst_elem_off[k], e_hi = c->inst_elem_off[k + 1], Ek = e_hi - e_lo;
            int begin = 0;
            for (int n = 0; n <= D; ++n) {
                const auto tab = nfaces(c->shape, n);
                const int stride = interior_dofs(c->shape, fe_degree, n);
                const int nfc = (int)tab.size();
                if (nfc == 0) continue;
                if (n < D) {
                    std::vector<Key> keys((size_t)Ek * nfc);
                    for (int64_t e = 0; e < Ek; ++e)
                        for (int f = 0; f < nfc; ++f) keys[e * nfc + f] = face_key(&c->hconn[(e_lo + e) * c->ngeom], tab[f]);
                    std::vector<int64_t> first, order;
                    group_faces(keys, first, order);
                    for (int64_t s = 0; s < Ek * nfc; ++s) {
                        const int64_t e = e_lo + s / nfc, f = s % nfc;
                        const int64_t s0 = first[s];
                        const int64_t e0 = e_lo + s0 / nfc, f0 = s0 % nfc;
                        for (int d = 0; d < stride; ++d) {
                            int64_t& dst = c->hedof[e * nf + begin + f * stride + d];
                            dst = (s0 == s) ? counter++ : c->hedof[e0 * nf + begin + f0 * stride + d];
                        }
                    }
                } else {
                    for (int64_t e = e_lo; e < e_hi; ++e)
                        for (int d = 0; d < nfc * stride; ++d) c->hedof[e * nf + begin + d] = counter++;
                }
                begin += nfc * stride;
            }
        }
        c->ndofobj = counter;
        c->inst_dof_off[c->ninst] = counter;
    }
    const size_t ndc = (size_t)c->ndofobj * ncomp;
    c->status.assign(ndc, 0);
    c->cval.assign(ndc, 0.0);
    c->hu.assign(ndc, 0.0);
    c->heq.assign(ndc, -1);
    c->numbered = false;
    c->u_nonzero = false;
    c->nnz = 0;
    c->pattern_ready = false;
    c->have64 = c->have32 = c->solved = false;
    // buffers sized by the previous field (a context reused for a new problem)
    c->dcval.release(); c->deq.release(); c->dstatus.release();
    c->inertia = false; c->nhist = 0; c->dhist.release(); c->nforce_w = 0;
    c->spmv_lpr64 = c->spmv_lpr32 = c->bspmv_lpb = 0;
    c->nbblocks = 0;
    c->mask_on = false;
    c->bsell_built = false;
    c->inst_iters.clear(); c->inst_relres.clear();
    c->blocked = false;
    if (n_dofobj) *n_dofobj = c->ndofobj;
    if (n_fun) *n_fun = nf;
    if (c->device < 0) return ISL_OK;
    std::vector<int32_t> soa;
    if (!on_device) {  // the device numbering leaves dedof on the device
        soa.resize((size_t)E * nf);
        for (int64_t e = 0; e < E; ++e)
            for (int f = 0; f < nf; ++f) soa[(size_t)f * E + e] = (int32_t)c->hedof[e * nf + f];
        ISL_CHECK_CUDA(c, c->dedof.alloc(soa.size()));
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dedof.p, soa.data(), soa.size() * 4, cudaMemcpyHostToDevice, c->stream));
    }
    ISL_CHECK_CUDA(c, c->du.alloc(ndc));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->du.p, 0, ndc * sizeof(double), c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    if (n_dofobj) *n_dofobj = c->ndofobj;
    if (n_fun) *n_fun = nf;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_field_elem_dofobj(isl_ctx* c, int64_t* out) {
    ISL_TRY
    if (!c || !c->fedeg || !out) return ISL_ERR_ARG;
    std::copy(c->hedof.begin(), c->hedof.end(), out);
    return ISL_OK;
    ISL_CATCH(c)
}

static int boundary_list(isl_ctx* c, std::vector<std::pair<int64_t, int>>& out) {
    if (c->bf_valid) { out = c->bf_cache; return ISL_OK; }
    const auto tab = nfaces(c->shape, c->dim - 1);
    const int nfc = (int)tab.size();
    const int64_t E = c->nelem;
    if (!c->host_setup && isl::device_setup_fits(c, nfc)) {
        isl::DeviceLevel lv;
        lv.nfc = nfc;
        lv.w = (int)tab[0].size();
        for (int f = 0; f < nfc; ++f)
            for (int i = 0; i < lv.w; ++i) lv.v[f][i] = tab[f][i];
        std::vector<int64_t> slots;
        cudaSetDevice(c->device);
        const int rc = isl::device_boundary_slots(c, lv, slots);
        if (rc != ISL_OK) return rc;
        out.resize(slots.size());
        for (size_t i = 0; i < slots.size(); ++i) out[i] = {slots[i] / nfc, (int)(slots[i] % nfc)};
        c->bf_cache = out;
        c->bf_valid = true;
        return ISL_OK;
    }
    std::vector<Key> keys((size_t)E * nfc);
    for (int64_t e = 0; e < E; ++e)
        for (int f = 0; f < nfc; ++f) keys[e * nfc + f] = face_key(&c->hconn[e * c->ngeom], tab[f]);
    std::vector<int64_t> first, order;
    group_faces(keys, first, order);
    out.clear();
    const int64_t n = (int64_t)order.size();
    int64_t i = 0;
    while (i < n) {
        int64_t j = i;
        while (j < n && keys[order[j]] == keys[order[i]]) ++j;
        if (j - i == 1) out.push_back({order[i] / nfc, (int)(order[i] % nfc)});
        i = j;
    }
    c->bf_cache = out;
    c->bf_valid = true;
    return ISL_OK;
}

int isl_boundary_faces(isl_ctx* c, int64_t* n, int64_t* elem, int* face) {
    ISL_TRY
    if (!c || !c->nelem || !n) return ISL_ERR_ARG;
    std::vector<std::pair<int64_t, int>> bf;
    const int rc = boundary_list(c, bf);
    if (rc != ISL_OK) return rc;
    *n = (int64_t)bf.size();
    if (elem && face)
        for (size_t i = 0; i < bf.size(); ++i) { elem[i] = bf[i].first; face[i] = bf[i].second; }
    return ISL_OK;
    ISL_CATCH(c)
}

// local FE positions on a boundary face: its vertices, interior DOFs of the
// element edges inside the face, and (3-D) the face's own interior DOFs
static std::vector<int> face_local_dofs(isl_ctx* c, int face) {
    const auto ftab = nfaces(c->shape, c->dim - 1);
    const std::vector<int>& fv = ftab[face];
    std::vector<int> out(fv.begin(), fv.end());
    if (c->fedeg == 1) return out;
    int begin = num_vertices(c->shape);
    const auto etab = nfaces(c->shape, 1);
    const int es = interior_dofs(c->shape, c->fedeg, 1);
    for (size_t ed = 0; ed < etab.size(); ++ed) {
        const bool in0 = std::find(fv.begin(), fv.end(), etab[ed][0]) != fv.end();
        const bool in1 = std::find(fv.begin(), fv.end(), etab[ed][1]) != fv.end();
        if (in0 && in1)
            for (int d = 0; d < es; ++d) out.push_back(begin + (int)ed * es + d);
    }
    begin += (int)etab.size() * es;
    if (c->dim == 3) {
        const int fs = interior_dofs(c->shape, c->fedeg, 2);
        for (int d = 0; d < fs; ++d) out.push_back(begin + face * fs + d);
    }
    return out;
}

int isl_boundary_points(isl_ctx* c, int64_t* n, double* x, int64_t* dofobj) {
    ISL_TRY
    if (!c || !c->fedeg || !n) return ISL_ERR_ARG;
    std::vector<std::pair<int64_t, int>> bf;
    const int brc = boundary_list(c, bf);
    if (brc != ISL_OK) return brc;
    // support points: FE nodes on the reference element
    std::vector<double> sup;
    {
        const int D = c->dim;
        if (c->shape == ISL_TET) {
            const double tv[10][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {.5, 0, 0},
                                      {.5, .5, 0}, {0, .5, 0}, {0, 0, .5}, {.5, 0, .5}, {0, .5, .5}};
            for (int i = 0; i < c->nfun; ++i) for (int d = 0; d < 3; ++d) sup.push_back(tv[i][d]);
        } else {
            const int k = c->fedeg, n1 = k + 1;
            const auto pos = cube_positions(D, k);
            sup.assign((size_t)c->nfun * D, 0.0);
            for (size_t m = 0; m < pos.size(); ++m) {
                int r = (int)m;
                for (int d = 0; d < D; ++d) { sup[pos[m] * D + d] = double(r % n1) / k; r /= n1; }
            }
        }
    }
    // geometry shape values at every local support point, and the local DOF
    // positions of every face, evaluated once
    std::vector<std::vector<double>> gv((size_t)c->nfun);
    int ng = 0;
    for (int l = 0; l < c->nfun; ++l) {
        std::vector<double> g;
        element_eval(c->shape, 1, &sup[(size_t)l * c->dim], gv[l], g, ng);
    }
    const int nfc = (int)nfaces(c->shape, c->dim - 1).size();
    std::vector<std::vector<int>> floc((size_t)nfc);
    for (int f = 0; f < nfc; ++f) floc[f] = face_local_dofs(c, f);
    int64_t cnt = 0;
    for (auto& ef : bf) {
        for (int l : floc[ef.second]) {
            if (x && dofobj) {
                const int64_t* ev = &c->hconn[ef.first * c->ngeom];
                for (int d = 0; d < c->dim; ++d) {
                    double s = 0.0;
                    for (int i = 0; i < ng; ++i) s += c->hX[ev[i] * c->dim + d] * gv[l][i];
                    x[cnt * c->dim + d] = s;
                }
                dofobj[cnt] = c->hedof[ef.first * c->nfun + l];
            }
            ++cnt;
        }
    }
    *n = cnt;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_constrain(isl_ctx* c, int64_t n, const int64_t* dofobj, const int* comp, const double* value) {
    ISL_TRY
    if (!c || !c->fedeg || (n > 0 && (!dofobj || !comp || !value))) return ISL_ERR_ARG;
    for (int64_t i = 0; i < n; ++i) {
        if (dofobj[i] < 0 || dofobj[i] >= c->ndofobj || comp[i] < 0 || comp[i] >= c->ncomp)
            ISL_FAIL(c, ISL_ERR_ARG, "constraint index out of range");
        const size_t k = (size_t)dofobj[i] * c->ncomp + comp[i];
        if (c->numbered && c->status[k] == 0) ISL_FAIL(c, ISL_ERR_ARG, "cannot constrain an active DOF after numbering");
        c->status[k] = 1;
        c->cval[k] = value[i];
    }
    if (c->dcval.p) {
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcval.p, c->cval.data(), c->cval.size() * 8, cudaMemcpyHostToDevice, c->stream));
        ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_scale_constraints(isl_ctx* c, double factor) {
    ISL_TRY
    if (!c || !c->fedeg) return ISL_ERR_ARG;
    for (size_t k = 0; k < c->status.size(); ++k) if (c->status[k]) c->cval[k] *= factor;
    if (c->dcval.p) {
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcval.p, c->cval.data(), c->cval.size() * 8, cudaMemcpyHostToDevice, c->stream));
        ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return ISL_OK;
    ISL_CATCH(c)
}

// consecutive numbering of ACTIVE components in DOF-object order
int isl_number_dofs(isl_ctx* c, int64_t* n_active) {
    ISL_TRY
    if (!c || !c->fedeg) return ISL_ERR_ARG;
    int64_t k = 0;
    c->inst_eq_off.assign(c->ninst + 1, 0);
    int64_t inst = 0;
    for (size_t i = 0; i < c->status.size(); ++i) {
        while (inst < c->ninst && (int64_t)i >= c->inst_dof_off[inst + 1] * c->ncomp) c->inst_eq_off[++inst] = k;
        c->heq[i] = c->status[i] == 0 ? (int32_t)k++ : -1;
    }
    while (inst < c->ninst) c->inst_eq_off[++inst] = k;
    if (k >= INT32_MAX) ISL_FAIL(c, ISL_ERR_ARG, "too many DOFs for 32-bit indices");
    c->neq = k;
    c->numbered = true;
    if (n_active) *n_active = k;
    c->nnz = 0;
    c->pattern_ready = false;
    c->nbblocks = 0;
    c->mask_on = false;
    c->bsell_built = false;
    if (c->device < 0) return ISL_OK;
    const size_t ndc = c->status.size();
    ISL_CHECK_CUDA(c, c->deq.alloc(ndc));
    ISL_CHECK_CUDA(c, c->dstatus.alloc(ndc));
    ISL_CHECK_CUDA(c, c->dcval.alloc(ndc));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->deq.p, c->heq.data(), ndc * 4, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dstatus.p, c->status.data(), ndc, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcval.p, c->cval.data(), ndc * 8, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    if (n_active) *n_active = k;
    c->nnz = 0;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_dof_index(isl_ctx* c, int64_t* out) {
    ISL_TRY
    if (!c || !c->numbered || !out) return ISL_ERR_ARG;
    for (size_t i = 0; i < c->heq.size(); ++i) out[i] = c->heq[i];
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_register_pattern(isl_ctx* c, int64_t* nnz) {
    ISL_TRY
    if (!c || !c->numbered) return ISL_ERR_ARG;
    if (c->device < 0) ISL_FAIL(c, ISL_ERR_ARG, "host-only context: the pattern is built on the device");
    cudaSetDevice(c->device);
    c->spmv_lpr64 = c->spmv_lpr32 = c->bspmv_lpb = 0;
    c->nbblocks = 0;
    c->mask_on = false;
    c->bsell_built = false;
    if (c->neq == 0) {  // every DOF constrained: an empty system, as the reference's Eigen3(0)
        c->nnz = 0;
        c->pattern_ready = true;
        c->blocked = false;
        if (nnz) *nnz = 0;
        return ISL_OK;
    }
    // elements with a constrained local DOF (Dirichlet lift candidates)
    std::vector<int32_t> lift;
    for (int64_t e = 0; e < c->nelem; ++e) {
        bool any = false;
        for (int f = 0; f < c->nfun && !any; ++f)
            for (int i = 0; i < c->ncomp; ++i)
                if (c->status[(size_t)c->hedof[e * c->nfun + f] * c->ncomp + i]) { any = true; break; }
        if (any) lift.push_back((int32_t)e);
    }
    c->n_lift = (int64_t)lift.size();
    ISL_CHECK_CUDA(c, c->dlift_elem.alloc(lift.size()));
    if (!lift.empty())
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dlift_elem.p, lift.data(), lift.size() * 4, cudaMemcpyHostToDevice, c->stream));
    int st = isl::pattern_build(c);
    if (st != ISL_OK) return st;
    c->pattern_ready = true;
    if (nnz) *nnz = c->nnz;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_laplace(isl_ctx* c, const double* kappa, int quad_degree) {
    ISL_TRY
    if (!c || !c->fedeg || !kappa) return ISL_ERR_ARG;
    if (c->ncomp != 1) ISL_FAIL(c, ISL_ERR_ARG, "Laplace needs a scalar field");
    c->kernel = ISL_KERNEL_LAPLACE;
    c->qdeg = quad_degree;
    c->stage_full = false;
    c->has_kqp = false;
    ISL_CHECK_CUDA(c, c->dcoef.alloc(c->nelem));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcoef.p, kappa, c->nelem * 8, cudaMemcpyHostToDevice, c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_laplace_qp(isl_ctx* c, const double* kappa, int quad_degree) {
    ISL_TRY
    if (!c || !c->fedeg || !kappa) return ISL_ERR_ARG;
    if (c->ncomp != 1) ISL_FAIL(c, ISL_ERR_ARG, "Laplace needs a scalar field");
    if (c->device < 0) ISL_FAIL(c, ISL_ERR_ARG, "host-only context");
    std::vector<double> w, xi;
    if (quad_degree < 1 || !quadrature(c->shape, quad_degree, w, xi)) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    const size_t nq = w.size(), E = (size_t)c->nelem;
    // [nelem][nq] (the order of isl_quadrature_points) -> [nq][nelem]
    std::vector<double> t(nq * E);
    for (size_t e = 0; e < E; ++e)
        for (size_t q = 0; q < nq; ++q) t[q * E + e] = kappa[e * nq + q];
    c->kernel = ISL_KERNEL_LAPLACE;
    c->qdeg = quad_degree;
    c->stage_full = false;
    ISL_CHECK_CUDA(c, c->dcoef.alloc(E));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dcoef.p, 0, E * 8, c->stream));
    ISL_CHECK_CUDA(c, c->dkqp.alloc(nq * E));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dkqp.p, t.data(), t.size() * 8, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    c->has_kqp = true;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_heat_static(isl_ctx* c, int material, const double* param, int quad_degree) {
    ISL_TRY
    if (!c || !c->fedeg || !param) return ISL_ERR_ARG;
    if (c->ncomp != 1) ISL_FAIL(c, ISL_ERR_ARG, "heat::Static needs a scalar field");
    if (material != ISL_THERMAL_CONSTANT && material != ISL_THERMAL_FENICS) ISL_FAIL(c, ISL_ERR_ARG, "thermal material");
    c->kernel = ISL_KERNEL_HEAT_STATIC;
    c->material = material;
    c->qdeg = quad_degree;
    c->stage_full = true;
    ISL_CHECK_CUDA(c, c->dcoef.alloc(c->nelem));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcoef.p, param, c->nelem * 8, cudaMemcpyHostToDevice, c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_history(isl_ctx* c, int nhist) {
    ISL_TRY
    if (!c || !c->fedeg || nhist < 0 || nhist > 4) ISL_FAIL(c, ISL_ERR_ARG, "isl_set_history: 0..4 past steps");
    if (c->device < 0) ISL_FAIL(c, ISL_ERR_ARG, "host-only context");
    cudaSetDevice(c->device);
    const size_t n = (size_t)c->ndofobj * c->ncomp;
    c->nhist = nhist;
    if (nhist == 0) { c->dhist.release(); return ISL_OK; }
    ISL_CHECK_CUDA(c, c->dhist.alloc(n * nhist));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dhist.p, 0, n * nhist * 8, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_push_history(isl_ctx* c) {
    ISL_TRY
    if (!c || !c->fedeg) return ISL_ERR_ARG;
    if (c->nhist == 0) ISL_FAIL(c, ISL_ERR_ARG, "isl_push_history: no history (isl_set_history)");
    cudaSetDevice(c->device);
    const int rc = isl::push_history_device(c);
    if (rc != ISL_OK) return rc;
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_inertia(isl_ctx* c, const double* density, double lhs_weight, int nweights, const double* weights) {
    ISL_TRY
    if (!c || !c->fedeg) return ISL_ERR_ARG;
    if (!density) { c->inertia = false; return ISL_OK; }
    if (nweights < 0 || nweights > 5 || nweights > c->nhist + 1 || (nweights > 0 && !weights))
        ISL_FAIL(c, ISL_ERR_ARG, "inertia terms: at most 5 weights and at most the stored history + 1");
    cudaSetDevice(c->device);
    ISL_CHECK_CUDA(c, c->drho.alloc(c->nelem));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->drho.p, density, c->nelem * 8, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    c->inertia = true;
    c->mass_w = lhs_weight;
    c->nhist_w = nweights;
    for (int k = 0; k < 5; ++k) c->hist_w[k] = k < nweights ? weights[k] : 0.0;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_force_history(isl_ctx* c, int nweights, const double* weights) {
    ISL_TRY
    if (!c || !c->fedeg) return ISL_ERR_ARG;
    if (nweights < 0 || nweights > 4 || nweights > c->nhist || (nweights > 0 && !weights))
        ISL_FAIL(c, ISL_ERR_ARG, "residual force history: at most 4 weights and at most the stored history");
    c->nforce_w = nweights;
    for (int k = 0; k < 4; ++k) c->force_w[k] = k < nweights ? weights[k] : 0.0;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_hyperelastic(isl_ctx* c, int material, const double* lambda, const double* mu, int quad_degree) {
    ISL_TRY
    if (!c || !c->fedeg || !lambda || !mu) return ISL_ERR_ARG;
    if (c->ncomp != c->dim) ISL_FAIL(c, ISL_ERR_ARG, "HyperElastic needs ncomp == dim");
    if (material != ISL_MAT_STVENANT && material != ISL_MAT_NEOHOOKE) ISL_FAIL(c, ISL_ERR_ARG, "material");
    c->kernel = ISL_KERNEL_HYPERELASTIC;
    c->material = material;
    c->stage_full = false;
    c->qdeg = quad_degree;
    ISL_CHECK_CUDA(c, c->dcoef.alloc(2 * c->nelem));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcoef.p, lambda, c->nelem * 8, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcoef.p + c->nelem, mu, c->nelem * 8, cudaMemcpyHostToDevice, c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_body_force_nodal(isl_ctx* c, const double* f) {
    ISL_TRY
    if (!c || !c->fedeg) return ISL_ERR_ARG;
    if (!f) { c->has_body = false; return ISL_OK; }
    ISL_CHECK_CUDA(c, c->dfnodal.alloc(c->nnodes * c->ncomp));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dfnodal.p, f, c->nnodes * c->ncomp * 8, cudaMemcpyHostToDevice, c->stream));
    c->has_body = true;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_neumann(isl_ctx* c, int64_t n, const int64_t* elem, const int* face, const double* traction, int squad_degree) {
    ISL_TRY
    return neumann_faces(c, n, elem, face, traction, false, squad_degree);
    ISL_CATCH(c)
}

int isl_set_neumann_vertex(isl_ctx* c, int64_t n, const int64_t* elem, const int* face, const double* traction,
                           int squad_degree) {
    ISL_TRY
    return neumann_faces(c, n, elem, face, traction, true, squad_degree);
    ISL_CATCH(c)
}

int isl_set_values(isl_ctx* c, const double* u) {
    ISL_TRY
    if (!c || !c->fedeg || !u) return ISL_ERR_ARG;
    const size_t n = (size_t)c->ndofobj * c->ncomp;
    c->u_nonzero = false;
    for (size_t i = 0; i < n; ++i) if (u[i] != 0.0) { c->u_nonzero = true; break; }
    if (c->device < 0) {  // host-only context: the values stay on the host (I/O)
        c->hu.assign(u, u + n);
        return ISL_OK;
    }
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->du.p, u, n * 8, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_get_values(isl_ctx* c, double* u) {
    ISL_TRY
    if (!c || !c->fedeg || !u) return ISL_ERR_ARG;
    const size_t n = (size_t)c->ndofobj * c->ncomp;
    if (c->device < 0) {
        if (c->hu.size() != n) return ISL_ERR_ARG;
        std::copy(c->hu.begin(), c->hu.end(), u);
        return ISL_OK;
    }
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(u, c->du.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_assemble(isl_ctx* c, int precision, int incremental, int with_residual) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    if (!c->pattern_ready || c->kernel < 0) ISL_FAIL(c, ISL_ERR_ARG, "assemble: pattern or kernel not set");
    if (precision < ISL_PREC_FP64 || precision > ISL_PREC_MIXED) ISL_FAIL(c, ISL_ERR_ARG, "precision");
    if (c->neq == 0) {
        c->have64 = precision != ISL_PREC_FP32;
        c->have32 = precision != ISL_PREC_FP64;
        c->solved = false;
        return ISL_OK;
    }
    cudaSetDevice(c->device);
    if (c->pattern_full != c->stage_full) {  // the kernel changed between symmetric and full staging
        const int st = isl::pattern_build(c);
        if (st != ISL_OK) return st;
    }
    return isl::assemble_device(c, precision, incremental, with_residual);
    ISL_CATCH(c)
}

int isl_solve(isl_ctx* c, int method, double tol, int64_t max_iter, int64_t* iters, double* rel_res) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    if (!c->pattern_ready || !(c->have64 || c->have32)) ISL_FAIL(c, ISL_ERR_ARG, "solve: nothing assembled");
    if (c->neq == 0) {
        c->solved = true;
        if (iters) *iters = 0;
        if (rel_res) *rel_res = 0.0;
        return ISL_OK;
    }
    if (method < ISL_SOLVE_CG_FP64 || method > ISL_SOLVE_BICGSTAB) ISL_FAIL(c, ISL_ERR_ARG, "solve: unknown method");
    if ((method == ISL_SOLVE_CG_FP64 || method == ISL_SOLVE_BICGSTAB) && !c->have64)
        ISL_FAIL(c, ISL_ERR_ARG, "solve: no FP64 matrix assembled");
    if (method == ISL_SOLVE_BICGSTAB && c->ninst > 1) ISL_FAIL(c, ISL_ERR_ARG, "solve: BiCGSTAB on one system only");
    if (method != ISL_SOLVE_BICGSTAB && c->stage_full)
        ISL_FAIL(c, ISL_ERR_ARG, "solve: the heat::Static tangent is not symmetric; use ISL_SOLVE_BICGSTAB");
    if (method == ISL_SOLVE_CG_FP32_IR && !c->have32)
        ISL_FAIL(c, ISL_ERR_ARG, "solve: the FP32 solve needs an FP32 matrix (ISL_PREC_MIXED or ISL_PREC_FP32)");
    if (!(tol >= 0.0)) ISL_FAIL(c, ISL_ERR_ARG, "tol");
    cudaSetDevice(c->device);
    return isl::solve_device(c, method, tol, max_iter, iters, rel_res);
    ISL_CATCH(c)
}

int isl_get_solution(isl_ctx* c, double* x) {
    ISL_TRY
    if (!c || !c->pattern_ready) return ISL_ERR_ARG;
    if (c->neq == 0) return ISL_OK;
    if (!x) return ISL_ERR_ARG;
    const double* src = c->solved ? c->dsol.p : c->drhs.p;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(x, src, c->neq * 8, cudaMemcpyDeviceToHost, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_get_rhs(isl_ctx* c, double* b) {
    ISL_TRY
    if (!c || !c->pattern_ready) return ISL_ERR_ARG;
    if (c->neq == 0) return ISL_OK;
    if (!b) return ISL_ERR_ARG;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(b, c->drhs.p, c->neq * 8, cudaMemcpyDeviceToHost, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_norm(isl_ctx* c, double* out) {
    ISL_TRY
    if (!c || !c->pattern_ready || !out) return ISL_ERR_ARG;
    if (c->neq == 0) { *out = 0.0; return ISL_OK; }
    if (c->device < 0) ISL_FAIL(c, ISL_ERR_ARG, "host-only context: no system");
    cudaSetDevice(c->device);
    if (c->ninst == 1) return isl::inst_norms_device(c, out);
    // one system made of the instances: sqrt(sum_k (N_k n_k)^2) / N
    std::vector<double> per((size_t)c->ninst);
    const int st = isl::inst_norms_device(c, per.data());
    if (st != ISL_OK) return st;
    double s = 0.0;
    for (int64_t k = 0; k < c->ninst; ++k) {
        const double nk = (double)(c->inst_eq_off[k + 1] - c->inst_eq_off[k]) * per[k];
        s += nk * nk;
    }
    *out = std::sqrt(s) / (double)c->neq;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_batch_norms(isl_ctx* c, double* out) {
    ISL_TRY
    if (!c || !c->pattern_ready || !out) return ISL_ERR_ARG;
    if (c->device < 0) ISL_FAIL(c, ISL_ERR_ARG, "host-only context: no system");
    if (c->neq == 0) { std::fill(out, out + c->ninst, 0.0); return ISL_OK; }
    cudaSetDevice(c->device);
    return isl::inst_norms_device(c, out);
    ISL_CATCH(c)
}

int isl_batch_scale_constraints(isl_ctx* c, const double* factors) {
    ISL_TRY
    if (!c || !c->fedeg || !factors) return ISL_ERR_ARG;
    if ((int64_t)c->inst_dof_off.size() != c->ninst + 1) ISL_FAIL(c, ISL_ERR_ARG, "no instances");
    // only the instances whose factor is not 1 change (and go to the device)
    for (int64_t k = 0; k < c->ninst; ++k) {
        if (factors[k] == 1.0) continue;
        const int64_t i0 = c->inst_dof_off[k] * c->ncomp, i1 = c->inst_dof_off[k + 1] * c->ncomp;
        for (int64_t i = i0; i < i1; ++i)
            if (c->status[i]) c->cval[i] *= factors[k];
        if (c->dcval.p && i1 > i0)
            ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dcval.p + i0, c->cval.data() + i0, (size_t)(i1 - i0) * 8,
                                              cudaMemcpyHostToDevice, c->stream));
    }
    if (c->dcval.p) ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_batch_set_mask(isl_ctx* c, const uint8_t* keep) {
    ISL_TRY
    if (!c || c->device < 0) return ISL_ERR_ARG;
    if (!keep) { c->mask_on = false; return ISL_OK; }
    if (c->ninst < 2) ISL_FAIL(c, ISL_ERR_ARG, "isl_batch_set_mask: a batch of instances only");
    cudaSetDevice(c->device);
    std::vector<int32_t> m((size_t)c->ninst);
    for (int64_t k = 0; k < c->ninst; ++k) m[k] = keep[k] ? 1 : 0;
    ISL_CHECK_CUDA(c, c->dinst_mask.alloc(m.size()));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dinst_mask.p, m.data(), m.size() * 4, cudaMemcpyHostToDevice, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    c->mask_on = true;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_distribute(isl_ctx* c, int add) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    if (!c->solved) ISL_FAIL(c, ISL_ERR_ARG, "distribute: no solution");
    cudaSetDevice(c->device);
    int st = (c->mask_on && c->ninst > 1) ? isl::distribute_masked(c, add) : isl::distribute_device(c, add);
    if (st == ISL_OK) c->u_nonzero = true;
    return st;
    ISL_CATCH(c)
}

int isl_quadrature_points(isl_ctx* c, int quad_degree, int64_t* n_points, double* x) {
    ISL_TRY
    if (!c || !c->fedeg || !n_points) return ISL_ERR_ARG;
    if (c->device < 0) ISL_FAIL(c, ISL_ERR_ARG, "host-only context: post-processing runs on the device");
    cudaSetDevice(c->device);
    return isl::quadrature_points_device(c, quad_degree, n_points, x);
    ISL_CATCH(c)
}

int isl_error_norm(isl_ctx* c, int order, int quad_degree, const double* ref, double* error) {
    ISL_TRY
    if (!c || !c->fedeg || !ref || !error || (order != 0 && order != 1)) return ISL_ERR_ARG;
    if (c->device < 0) ISL_FAIL(c, ISL_ERR_ARG, "host-only context: post-processing runs on the device");
    cudaSetDevice(c->device);
    return isl::error_norm_device(c, order, quad_degree, ref, error);
    ISL_CATCH(c)
}

int isl_get_csr(isl_ctx* c, int64_t* rowptr, int64_t* colind, double* values) {
    ISL_TRY
    if (!c || !c->pattern_ready) return ISL_ERR_ARG;
    if (c->neq == 0) {
        if (rowptr) rowptr[0] = 0;
        return ISL_OK;
    }
    if (rowptr) {
        std::vector<int32_t> t(c->neq + 1);
        ISL_CHECK_CUDA(c, cudaMemcpy(t.data(), c->drowptr.p, t.size() * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < t.size(); ++i) rowptr[i] = t[i];
    }
    if (colind) {
        std::vector<int32_t> t(c->nnz);
        ISL_CHECK_CUDA(c, cudaMemcpy(t.data(), c->dcolind.p, t.size() * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < t.size(); ++i) colind[i] = t[i];
    }
    if (values) {
        if (c->have64) {
            ISL_CHECK_CUDA(c, cudaMemcpy(values, c->dval64.p, c->nnz * 8, cudaMemcpyDeviceToHost));
        } else if (c->have32) {
            std::vector<float> t(c->nnz);
            ISL_CHECK_CUDA(c, cudaMemcpy(t.data(), c->dval32.p, t.size() * 4, cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < t.size(); ++i) values[i] = t[i];
        } else {
            ISL_FAIL(c, ISL_ERR_ARG, "no values assembled");
        }
    }
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_sync(isl_ctx* c) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_timing(isl_ctx* c, int on) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    c->timing = on != 0;
    for (int i = 0; i < ISL_NTIMERS; ++i) { c->tms[i] = 0; c->tcount[i] = 0; }
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_timings(isl_ctx* c, double* ms, int64_t* counts) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    for (int i = 0; i < ISL_NTIMERS; ++i) {
        if (ms) ms[i] = c->tms[i];
        if (counts) counts[i] = c->tcount[i];
    }
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_time_spmv(isl_ctx* c, int precision, int nrep, double* ms) {
    ISL_TRY
    if (!c || !c->pattern_ready || c->neq == 0 || !ms || nrep == 0) return ISL_ERR_ARG;
    return isl::time_spmv(c, precision, nrep, ms);
    ISL_CATCH(c)
}

int isl_mark(isl_ctx* c, int slot) {
    ISL_TRY
    if (!c || c->device < 0 || slot < 0 || slot >= 8) return ISL_ERR_ARG;
    ISL_CHECK_CUDA(c, cudaEventRecord(c->mark[slot], c->stream));
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_elapsed(isl_ctx* c, int a, int b, double* ms) {
    ISL_TRY
    if (!c || c->device < 0 || a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) return ISL_ERR_ARG;
    ISL_CHECK_CUDA(c, cudaEventSynchronize(c->mark[b]));
    float t = 0.f;
    ISL_CHECK_CUDA(c, cudaEventElapsedTime(&t, c->mark[a], c->mark[b]));
    *ms = t;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_launch_count(isl_ctx* c, int64_t* n) {
    ISL_TRY
    if (!c || !n) return ISL_ERR_ARG;
    *n = c->launches;
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_set_option(isl_ctx* c, int key, int64_t value) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    if (key == ISL_OPT_BLOCK_SOLVER) { c->use_block = value != 0; return ISL_OK; }
    if (key == ISL_OPT_BATCHED_SOLVE) { c->force_batched = value != 0; return ISL_OK; }
    if (key == ISL_OPT_FOLD_DIRECTION) { c->fuse_dir = value != 0; return ISL_OK; }
    if (key == ISL_OPT_SHORT_COLUMNS) { c->use_scol16 = value != 0; return ISL_OK; }
    if (key == ISL_OPT_SHARED_GEOMETRY) { c->use_shared_geo = value != 0; return ISL_OK; }
    if (key == ISL_OPT_RELIABLE_DROP) {
        if (value < 1 || value > 8) ISL_FAIL(c, ISL_ERR_ARG, "ISL_OPT_RELIABLE_DROP takes 1..8");
        c->ru_drop2 = std::pow(10.0, -(double)value);
        return ISL_OK;
    }
    if (key == ISL_OPT_BLOCK_UPDATE) {
        if (value != 0 && !isl::update_kind_valid((int)value))
            ISL_FAIL(c, ISL_ERR_ARG, "ISL_OPT_BLOCK_UPDATE takes 0, 1, 2, 4 or 8");
        c->bupd_kind[0] = c->bupd_kind[1] = (int)value;
        return ISL_OK;
    }
    if (key == ISL_OPT_BARRIER_TEST) { c->barrier_test = value != 0; return ISL_OK; }
    if (key == ISL_OPT_PERSISTENT) {
        if (value < 0 || value > 2) ISL_FAIL(c, ISL_ERR_ARG, "ISL_OPT_PERSISTENT takes 0, 1 or 2");
        c->use_persist = (int)value;
        return ISL_OK;
    }
    if (key == ISL_OPT_BICGSTAB_KIND) {
        if (value < 0 || value > 108 || !isl::bicgstab_kind_valid(c, (int)value))
            ISL_FAIL(c, ISL_ERR_ARG, "ISL_OPT_BICGSTAB_KIND: 0, CSR lanes per row 2..16, or 102/104/108 with a sliced-ELL copy");
        c->bicg_forced = (int)value;
        return ISL_OK;
    }
    if (key == ISL_OPT_HOST_SETUP) {
        c->host_setup = value != 0;
        c->bf_valid = false;
        c->bf_cache.clear();
        return ISL_OK;
    }
    if (key == ISL_OPT_SPMV32_KIND) {
        if (value < 0 || value > 108 || !isl::spmv32_kind_valid(c, (int)value))
            ISL_FAIL(c, ISL_ERR_ARG, "ISL_OPT_SPMV32_KIND: 0, CSR lanes per row 2..32, or 102/104/108 with a sliced-ELL copy");
        c->spmv32_forced = (int)value;
        c->spmv_lpr32 = (int)value;
        return ISL_OK;
    }
    ISL_FAIL(c, ISL_ERR_ARG, "unknown or read-only option");
    ISL_CATCH(c)
}

int isl_get_option(isl_ctx* c, int key, int64_t* value) {
    ISL_TRY
    if (!c || !value) return ISL_ERR_ARG;
    if (key == ISL_OPT_BLOCK_SOLVER) { *value = c->use_block; return ISL_OK; }
    if (key == ISL_OPT_BATCHED_SOLVE) { *value = c->force_batched; return ISL_OK; }
    if (key == ISL_OPT_FOLD_DIRECTION) { *value = c->fuse_dir; return ISL_OK; }
    if (key == ISL_OPT_SHORT_COLUMNS) {
        *value = c->use_scol16 && (c->blocked ? c->scol16 : c->ss16) ? 1 : 0;
        return ISL_OK;
    }
    if (key == ISL_OPT_RELIABLE_DROP) { *value = (int64_t)std::lround(-std::log10(c->ru_drop2)); return ISL_OK; }
    if (key == ISL_OPT_SHARED_GEOMETRY) { *value = c->last_shared_geo ? 1 : 0; return ISL_OK; }
    if (key == ISL_OPT_BLOCK_UPDATE) { *value = c->bupd_kind[c->fuse_dir ? 1 : 0]; return ISL_OK; }
    if (key == ISL_OPT_DIRECT_BLOCKS) { *value = c->last_direct; return ISL_OK; }
    if (key == ISL_OPT_TUNE_RUNS) { *value = c->tune_runs; return ISL_OK; }
    if (key == ISL_OPT_ELEM_VARIANT) { *value = c->elem_variant; return ISL_OK; }
    if (key == ISL_OPT_PERSISTENT) { *value = c->use_persist; return ISL_OK; }
    if (key == ISL_OPT_BLOCKED) { *value = c->blocked ? (c->bpad ? 2 : 1) : 0; return ISL_OK; }
    if (key == ISL_OPT_NBLOCKS) { *value = c->blocked ? c->nblk : 0; return ISL_OK; }
    if (key == ISL_OPT_NSLOTS) { *value = c->blocked ? c->nslot : 0; return ISL_OK; }
    if (key == ISL_OPT_SPMV32_KIND) { *value = c->spmv_lpr32; return ISL_OK; }
    if (key == ISL_OPT_HOST_SETUP) { *value = c->host_setup; return ISL_OK; }
    if (key == ISL_OPT_BICGSTAB_KIND) { *value = c->bicg_lpr; return ISL_OK; }
    if (key == ISL_OPT_SCALAR_SLOTS) { *value = c->ss_nslot; return ISL_OK; }
    ISL_FAIL(c, ISL_ERR_ARG, "unknown option");
    ISL_CATCH(c)
}

int isl_quadrature_rule(int shape, int degree, int* n, double* w, double* xi) {
    ISL_TRY
    // the reference's rules exist for DEGREE > 0 only (base/quad/GaussLegendre.hpp:61,
    // base/quad/GaussTetrahedron.hpp:93-175)
    if (!n || degree < 1 || !(shape == ISL_QUAD || shape == ISL_TET || shape == ISL_HEX || shape == ISL_TRI))
        return ISL_ERR_ARG;
    std::vector<double> ww, xx;
    if (!quadrature(shape, degree, ww, xx)) return ISL_ERR_ARG;
    *n = (int)ww.size();
    if (w) std::copy(ww.begin(), ww.end(), w);
    if (xi) std::copy(xx.begin(), xx.end(), xi);
    return ISL_OK;
    ISL_CATCH(nullptr)
}

int isl_device_memory(int device, int64_t* free_bytes, int64_t* total_bytes) {
    ISL_TRY
    if (!free_bytes || !total_bytes) return ISL_ERR_ARG;
    int cur = 0;
    cudaGetDevice(&cur);
    if (cudaSetDevice(device) != cudaSuccess) return ISL_ERR_CUDA;
    size_t f = 0, t = 0;
    const cudaError_t e = cudaMemGetInfo(&f, &t);
    cudaSetDevice(cur);
    if (e != cudaSuccess) return ISL_ERR_CUDA;
    *free_bytes = (int64_t)f;
    *total_bytes = (int64_t)t;
    return ISL_OK;
    ISL_CATCH(nullptr)
}

int isl_batch_info(isl_ctx* c, int64_t* n_inst, int64_t* eq_off, int64_t* dofobj_off) {
    ISL_TRY
    if (!c) return ISL_ERR_ARG;
    if (n_inst) *n_inst = c->ninst;
    if (eq_off) {
        if (!c->numbered) ISL_FAIL(c, ISL_ERR_ARG, "batch info: DOFs not numbered");
        std::copy(c->inst_eq_off.begin(), c->inst_eq_off.end(), eq_off);
    }
    if (dofobj_off) {
        if (!c->fedeg) ISL_FAIL(c, ISL_ERR_ARG, "batch info: no field");
        std::copy(c->inst_dof_off.begin(), c->inst_dof_off.end(), dofobj_off);
    }
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_batch_solve_stats(isl_ctx* c, int64_t* iters, double* rel_res) {
    ISL_TRY
    if (!c || c->inst_iters.empty()) return ISL_ERR_ARG;
    for (int64_t k = 0; k < c->ninst; ++k) {
        if (iters) iters[k] = c->inst_iters[k];
        if (rel_res) rel_res[k] = c->inst_relres[k];
    }
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_time_kernels(isl_ctx* c, int nrep, double* ms) {
    ISL_TRY
    if (!c || !c->pattern_ready || c->neq == 0 || !ms || nrep <= 0) return ISL_ERR_ARG;
    cudaSetDevice(c->device);
    return isl::time_kernels(c, nrep, ms);
    ISL_CATCH(c)
}

}  // extern "C"
