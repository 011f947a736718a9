// Smoothed-aggregation AMG set-up on the host (Vanek, Mandel and Brezina, "Algebraic multigrid by
// smoothed aggregation for second and fourth order elliptic problems", Computing 56, 1996), with the
// choices of the AMGCL configuration the reference uses (amg<smoothed_aggregation, spai0>):
// - strength of connection: j is strongly connected to i when a_ij^2 > eps^2 |a_ii a_jj|, eps = 0.08 on
//   the finest level and halved on every coarser one;
// - plain aggregation: a node whose strong neighbours are all free roots an aggregate of itself and
//   them; every node left joins the aggregate of a strongly connected aggregated neighbour (or roots
//   its own); a node without strong connections belongs to no aggregate (the smoother treats it);
// - tentative prolongation: the constant vector on each aggregate;
// - prolongation smoothing: P = (I - omega D_f^-1 A_f) P_tent with the filtered matrix A_f (weak
//   connections lumped onto the diagonal) and omega = (4/3) relax / rho(D_f^-1 A_f), rho bounded by
//   the largest absolute row sum of D_f^-1 A_f;
// - restriction R = P^T and Galerkin coarse operators A_c = R A P;
// - SPAI-0 smoothing, m_i = a_ii / sum_j a_ij^2;
// - the coarsest level (at most coarse_enough unknowns) solved with a dense inverse.
#include "amg.h"

#include <algorithm>
#include <cmath>

namespace opg {
namespace {

std::vector<double> diagonal(const HostCsr& A) {
    std::vector<double> d((size_t) A.n, 0.);
    for (long long i = 0; i < A.n; ++i)
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
            if (A.col[q] == i) d[i] += A.val[q];
    return d;
}

HostCsr transpose(const HostCsr& A) {
    HostCsr T;
    T.n = A.m;
    T.m = A.n;
    T.ptr.assign((size_t) T.n + 1, 0);
    for (int c : A.col) T.ptr[(size_t) c + 1]++;
    for (long long i = 0; i < T.n; ++i) T.ptr[i + 1] += T.ptr[i];
    T.col.resize(A.col.size());
    T.val.resize(A.val.size());
    std::vector<long long> pos(T.ptr.begin(), T.ptr.end() - 1);
    for (long long i = 0; i < A.n; ++i)
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
            const long long w = pos[A.col[q]]++;
            T.col[w] = (int) i;
            T.val[w] = A.val[q];
        }
    return T;
}

// C = A B (rows of C in column order)
HostCsr multiply(const HostCsr& A, const HostCsr& B) {
    HostCsr C;
    C.n = A.n;
    C.m = B.m;
    C.ptr.assign((size_t) C.n + 1, 0);
    std::vector<long long> mark((size_t) B.m, -1);
    std::vector<double> acc((size_t) B.m, 0.);
    std::vector<int> cols;
    for (long long i = 0; i < A.n; ++i) {
        cols.clear();
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
            const int k = A.col[q];
            const double a = A.val[q];
            for (long long t = B.ptr[k]; t < B.ptr[k + 1]; ++t) {
                const int j = B.col[t];
                if (mark[j] != i) {
                    mark[j] = i;
                    acc[j] = 0.;
                    cols.push_back(j);
                }
                acc[j] += a * B.val[t];
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int j : cols) {
            C.col.push_back(j);
            C.val.push_back(acc[j]);
        }
        C.ptr[i + 1] = (long long) C.col.size();
    }
    return C;
}

// strong[q] for every entry q of A (off-diagonal only)
std::vector<char> strength(const HostCsr& A, const std::vector<double>& dia, double eps) {
    std::vector<char> s(A.col.size(), 0);
    const double e2 = eps * eps;
    for (long long i = 0; i < A.n; ++i)
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
            const int j = A.col[q];
            if (j == i) continue;
            const double v = A.val[q];
            s[q] = v * v > e2 * std::fabs(dia[i] * dia[j]);
        }
    return s;
}

// plain aggregation; returns the number of aggregates (agg[i] = -1: no aggregate)
long long aggregate(const HostCsr& A, const std::vector<char>& strong, std::vector<long long>& agg) {
    const long long n = A.n;
    const long long UNDECIDED = -2;
    agg.assign((size_t) n, UNDECIDED);
    for (long long i = 0; i < n; ++i) {
        bool any = false;
        for (long long q = A.ptr[i]; q < A.ptr[i + 1] && !any; ++q) any = strong[q];
        if (!any) agg[i] = -1;
    }
    long long na = 0;
    for (long long i = 0; i < n; ++i) {
        if (agg[i] != UNDECIDED) continue;
        bool free = true;
        for (long long q = A.ptr[i]; q < A.ptr[i + 1] && free; ++q)
            if (strong[q] && agg[A.col[q]] != UNDECIDED) free = false;
        if (!free) continue;
        agg[i] = na;
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
            if (strong[q]) agg[A.col[q]] = na;
        ++na;
    }
    for (long long i = 0; i < n; ++i) {
        if (agg[i] != UNDECIDED) continue;
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
            if (strong[q] && agg[A.col[q]] >= 0) {
                agg[i] = agg[A.col[q]];
                break;
            }
        if (agg[i] == UNDECIDED) agg[i] = na++;
    }
    return na;
}

// the smoothed prolongation of one level
HostCsr prolongation(const HostCsr& A, const std::vector<double>& dia, const std::vector<char>& strong, const std::vector<long long>& agg, long long na,
                     double relax) {
    const long long n = A.n;
    // filtered diagonal: weak off-diagonal entries lumped onto it
    std::vector<double> df(dia);
    for (long long i = 0; i < n; ++i)
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
            if (A.col[q] != i && !strong[q]) df[i] += A.val[q];
    // rho(D_f^-1 A_f) <= max_i sum_j |af_ij| / |df_i|
    double rho = 0.;
    for (long long i = 0; i < n; ++i) {
        if (df[i] == 0.) continue;
        double s = std::fabs(df[i]);
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
            if (A.col[q] != i && strong[q]) s += std::fabs(A.val[q]);
        rho = std::max(rho, s / std::fabs(df[i]));
    }
    const double omega = rho > 0. ? relax * (4.0 / 3.0) / rho : 0.;
    HostCsr P;
    P.n = n;
    P.m = na;
    P.ptr.assign((size_t) n + 1, 0);
    std::vector<long long> mark((size_t) na, -1);
    std::vector<double> acc((size_t) na, 0.);
    std::vector<int> cols;
    for (long long i = 0; i < n; ++i) {
        cols.clear();
        auto add = [&](long long a, double v) {
            if (a < 0) return;
            if (mark[a] != i) {
                mark[a] = i;
                acc[a] = 0.;
                cols.push_back((int) a);
            }
            acc[a] += v;
        };
        add(agg[i], 1.0);
        if (df[i] != 0.) {
            const double s = omega / df[i];
            add(agg[i], -s * df[i]);
            for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
                const int j = A.col[q];
                if (j != i && strong[q]) add(agg[j], -s * A.val[q]);
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int a : cols)
            if (acc[a] != 0.) {
                P.col.push_back(a);
                P.val.push_back(acc[a]);
            }
        P.ptr[i + 1] = (long long) P.col.size();
    }
    return P;
}

std::vector<double> spai0(const HostCsr& A, const std::vector<double>& dia) {
    std::vector<double> M((size_t) A.n, 0.);
    for (long long i = 0; i < A.n; ++i) {
        double s = 0.;
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q) s += A.val[q] * A.val[q];
        M[i] = s > 0. ? dia[i] / s : 0.;
    }
    return M;
}

// dense inverse by Gauss-Jordan elimination with partial pivoting; a pivot below 1e-14 of the
// matrix's largest entry (a singular coarse operator) leaves its row and column of the inverse at 0
std::vector<double> dense_inverse(const HostCsr& A) {
    const long long n = A.n;
    std::vector<double> a((size_t) (n * n), 0.), inv((size_t) (n * n), 0.);
    double amax = 0.;
    for (long long i = 0; i < n; ++i)
        for (long long q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
            a[(size_t) (i * n + A.col[q])] += A.val[q];
            amax = std::max(amax, std::fabs(A.val[q]));
        }
    for (long long i = 0; i < n; ++i) inv[(size_t) (i * n + i)] = 1.;
    std::vector<char> dead((size_t) n, 0);
    for (long long c = 0; c < n; ++c) {
        long long piv = c;
        for (long long r = c + 1; r < n; ++r)
            if (std::fabs(a[(size_t) (r * n + c)]) > std::fabs(a[(size_t) (piv * n + c)])) piv = r;
        if (std::fabs(a[(size_t) (piv * n + c)]) <= 1e-14 * amax) {
            dead[c] = 1;
            continue;
        }
        if (piv != c)
            for (long long k = 0; k < n; ++k) {
                std::swap(a[(size_t) (c * n + k)], a[(size_t) (piv * n + k)]);
                std::swap(inv[(size_t) (c * n + k)], inv[(size_t) (piv * n + k)]);
            }
        const double d = 1.0 / a[(size_t) (c * n + c)];
        for (long long k = 0; k < n; ++k) {
            a[(size_t) (c * n + k)] *= d;
            inv[(size_t) (c * n + k)] *= d;
        }
        for (long long r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = a[(size_t) (r * n + c)];
            if (f == 0.) continue;
            for (long long k = 0; k < n; ++k) {
                a[(size_t) (r * n + k)] -= f * a[(size_t) (c * n + k)];
                inv[(size_t) (r * n + k)] -= f * inv[(size_t) (c * n + k)];
            }
        }
    }
    for (long long c = 0; c < n; ++c)
        if (dead[c])
            for (long long k = 0; k < n; ++k) inv[(size_t) (c * n + k)] = inv[(size_t) (k * n + c)] = 0.;
    return inv;
}

}  // namespace

int amg_build_host(const HostCsr& A0, const AmgParams& prm, AmgHost* out) {
    if (A0.n <= 0 || A0.n != A0.m || (long long) A0.ptr.size() != A0.n + 1) return fail(OPFLOW_E_INVALID, "AMG: the matrix must be square CSR");
    out->levels.clear();
    HostCsr A = A0;
    double eps = prm.eps_strong;
    for (int lev = 0;; ++lev) {
        AmgLevelHost L;
        const std::vector<double> dia = diagonal(A);
        L.M = spai0(A, dia);
        if (A.n <= prm.coarse_enough || lev + 1 >= prm.max_levels) {
            L.A = std::move(A);
            out->levels.push_back(std::move(L));
            break;
        }
        const std::vector<char> strong = strength(A, dia, eps);
        std::vector<long long> agg;
        const long long na = aggregate(A, strong, agg);
        if (na == 0 || na >= A.n) {  // no coarsening possible: this level is the coarsest
            L.A = std::move(A);
            out->levels.push_back(std::move(L));
            break;
        }
        L.P = prolongation(A, dia, strong, agg, na, prm.relax);
        L.R = transpose(L.P);
        HostCsr Ac = multiply(L.R, multiply(A, L.P));
        L.A = std::move(A);
        out->levels.push_back(std::move(L));
        A = std::move(Ac);
        eps *= 0.5;
    }
    const HostCsr& C = out->levels.back().A;
    if (C.n > 3000) return fail(OPFLOW_E_UNSUPPORTED, "AMG: coarsening stalled at %lld unknowns", C.n);
    out->coarse_inv = dense_inverse(C);
    return OPFLOW_OK;
}

}  // namespace opg
