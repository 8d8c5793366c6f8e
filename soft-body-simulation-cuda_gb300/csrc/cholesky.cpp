// Sparse Cholesky of the scalar PD system (host side): ordering, symbolic
// analysis, FP64 supernodal multifrontal factorisation and the per-supernode
// M_s blocks of the GPU triangular solves.  See cholesky.h.
#include "cholesky.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <set>
#include <string>

#include "engine.h"

namespace pdgb {

// ------------------------------------------------------------ assembly
SparseSym assemble_system(int nv, int nt, const uint32_t* tets4, const double* dminv, const double* coef,
                          const std::vector<double>& mdt2) {
    // count neighbours per row (with duplicates), then sort/merge per row
    std::vector<int64_t> cnt(nv + 1, 0);
    for (int t = 0; t < nt; ++t)
        for (int a = 0; a < 4; ++a) cnt[tets4[4 * (size_t)t + a] + 1] += 4;
    for (int v = 0; v < nv; ++v) cnt[v + 1] += cnt[v] + 1;  // + diagonal
    std::vector<int> ci(cnt[nv]);
    std::vector<double> cx(cnt[nv]);
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int v = 0; v < nv; ++v) {
        ci[fill[v]] = v;
        cx[fill[v]++] = mdt2[v];
    }
    for (int t = 0; t < nt; ++t) {
        const double* D = dminv + 9 * (size_t)t;
        double B[3][4];
        for (int r = 0; r < 3; ++r) {
            B[r][1] = D[0 * 3 + r];
            B[r][2] = D[1 * 3 + r];
            B[r][3] = D[2 * 3 + r];
            B[r][0] = -(B[r][1] + B[r][2] + B[r][3]);
        }
        const uint32_t* id = tets4 + 4 * (size_t)t;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) {
                const double s = coef[t] * (B[0][a] * B[0][b] + B[1][a] * B[1][b] + B[2][a] * B[2][b]);
                ci[fill[id[a]]] = (int)id[b];
                cx[fill[id[a]]++] = s;
            }
    }
    SparseSym K;
    K.n = nv;
    K.p.assign(nv + 1, 0);
    K.i.reserve(cnt[nv] / 2);
    K.x.reserve(cnt[nv] / 2);
    std::vector<std::pair<int, double>> row;
    for (int v = 0; v < nv; ++v) {
        row.clear();
        for (int64_t e = cnt[v]; e < cnt[v + 1]; ++e) row.push_back({ci[e], cx[e]});
        std::sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        int last = -1;
        for (auto& e : row) {
            if (e.first == last) K.x.back() += e.second;
            else {
                K.i.push_back(e.first);
                K.x.push_back(e.second);
                last = e.first;
            }
        }
        K.p[v + 1] = (int64_t)K.i.size();
    }
    return K;
}

SparseSym layout_system(const HostLayout& L) {
    std::vector<double> mdt2(L.nv);
    for (int i = 0; i < L.nv; ++i) mdt2[i] = (double)L.coef[i].x;
    return assemble_system(L.nv, L.nt, L.tets_int.data(), L.dminv_d.data(), L.coef_d.data(), mdt2);
}

std::vector<float> layout_xyz(const HostLayout& L) {
    std::vector<float> xyz(3 * (size_t)L.nv);
    for (int i = 0; i < L.nv; ++i) {
        xyz[3 * (size_t)i] = L.x0[i].x;
        xyz[3 * (size_t)i + 1] = L.x0[i].y;
        xyz[3 * (size_t)i + 2] = L.x0[i].z;
    }
    return xyz;
}

// ------------------------------------------------------------------ AMD
std::vector<int> amd_order(const SparseSym& A) {
    const int n = A.n;
    enum : char { VAR = 0, ELEM = 1, DEAD = 2, MERGED = 3 };
    std::vector<std::vector<int>> vars(n), elems(n), Le(n), merged(n);
    std::vector<char> state(n, VAR);
    std::vector<int> nv(n, 1), deg(n, 0), mark(n, 0), tmpdeg(n, 0);
    std::vector<long long> w(n, 0);
    for (int i = 0; i < n; ++i) {
        for (int64_t e = A.p[i]; e < A.p[i + 1]; ++e)
            if (A.i[e] != i) vars[i].push_back(A.i[e]);
        deg[i] = (int)vars[i].size();
    }
    std::vector<int> head(n + 1, -1), nxt(n, -1), prv(n, -1);
    auto ins = [&](int i) {
        const int d = deg[i];
        nxt[i] = head[d];
        prv[i] = -1;
        if (head[d] >= 0) prv[head[d]] = i;
        head[d] = i;
    };
    auto rem = [&](int i) {
        if (prv[i] >= 0) nxt[prv[i]] = nxt[i];
        else head[deg[i]] = nxt[i];
        if (nxt[i] >= 0) prv[nxt[i]] = prv[i];
        nxt[i] = prv[i] = -1;
    };
    for (int i = 0; i < n; ++i) ins(i);
    int k = 0, mindeg = 0, stamp = 0;
    long long wflg = 1;
    std::vector<int> order;
    order.reserve(n);
    std::vector<int> Lp, keep;
    std::vector<std::pair<uint64_t, int>> hashed;
    while (k < n) {
        while (mindeg <= n && head[mindeg] < 0) ++mindeg;
        if (mindeg > n) break;  // cannot happen while k < n
        const int p = head[mindeg];
        rem(p);
        int nvp = nv[p];
        // ---- new element p: Lp = A_p U (U_{e in E_p} L_e) \ {p}; absorb E_p
        ++stamp;
        mark[p] = stamp;
        Lp.clear();
        for (int j : vars[p])
            if (state[j] == VAR && mark[j] != stamp) {
                mark[j] = stamp;
                Lp.push_back(j);
            }
        for (int e : elems[p])
            if (state[e] == ELEM) {
                for (int j : Le[e])
                    if (state[j] == VAR && mark[j] != stamp) {
                        mark[j] = stamp;
                        Lp.push_back(j);
                    }
                state[e] = DEAD;
                std::vector<int>().swap(Le[e]);
            }
        std::vector<int>().swap(vars[p]);
        std::vector<int>().swap(elems[p]);
        state[p] = ELEM;
        for (int j : Lp) rem(j);
        // ---- |L_e \ L_p| for every element adjacent to L_p (w trick)
        for (int i : Lp)
            for (int e : elems[i]) {
                if (state[e] != ELEM) continue;
                if (w[e] < wflg) {
                    // first touch this round: prune and weigh L_e
                    auto& L = Le[e];
                    size_t q = 0;
                    long long sz = 0;
                    for (int j : L)
                        if (state[j] == VAR) {
                            L[q++] = j;
                            sz += nv[j];
                        }
                    L.resize(q);
                    w[e] = wflg + sz;
                }
                w[e] -= nv[i];
            }
        // ---- prune lists, aggressive absorption, mass elimination
        keep.clear();
        for (int i : Lp) {
            auto& E = elems[i];
            size_t q = 0;
            long long de = 0;
            for (int e : E) {
                if (state[e] != ELEM) continue;
                const long long we = w[e] - wflg;
                if (we <= 0) {  // L_e inside L_p: absorb e into p
                    state[e] = DEAD;
                    std::vector<int>().swap(Le[e]);
                } else {
                    de += we;
                    E[q++] = e;
                }
            }
            E.resize(q);
            auto& Av = vars[i];
            q = 0;
            long long da = 0;
            for (int j : Av)
                if (state[j] == VAR && mark[j] != stamp) {
                    da += nv[j];
                    Av[q++] = j;
                }
            Av.resize(q);
            if (E.empty() && Av.empty()) {  // adjacent to p only: eliminate with p
                state[i] = MERGED;
                merged[p].push_back(i);
                nvp += nv[i];
                nv[i] = 0;
                continue;
            }
            tmpdeg[i] = (int)std::min<long long>(de + da, n);
            E.insert(E.begin(), p);
            keep.push_back(i);
        }
        // ---- supervariables: identical (E_i, A_i) lists
        hashed.clear();
        for (int i : keep) {
            uint64_t h = 1469598103934665603ULL;
            uint64_t s = 0;
            for (int e : elems[i]) s += (uint64_t)e * 2654435761ULL;
            for (int j : vars[i]) s += (uint64_t)j * 40503ULL + 7;
            h ^= s + ((uint64_t)elems[i].size() << 40) + ((uint64_t)vars[i].size() << 20);
            hashed.push_back({h, i});
        }
        std::sort(hashed.begin(), hashed.end());
        for (size_t a = 0; a < hashed.size();) {
            size_t b = a + 1;
            while (b < hashed.size() && hashed[b].first == hashed[a].first) ++b;
            if (b - a > 1) {
                for (size_t x = a; x < b; ++x) {
                    const int i = hashed[x].second;
                    if (state[i] != VAR) continue;
                    std::vector<int> ei(elems[i]), vi(vars[i]);
                    std::sort(ei.begin(), ei.end());
                    std::sort(vi.begin(), vi.end());
                    for (size_t y = x + 1; y < b; ++y) {
                        const int j = hashed[y].second;
                        if (state[j] != VAR) continue;
                        if (elems[j].size() != ei.size() || vars[j].size() != vi.size()) continue;
                        std::vector<int> ej(elems[j]), vj(vars[j]);
                        std::sort(ej.begin(), ej.end());
                        std::sort(vj.begin(), vj.end());
                        if (ej == ei && vj == vi) {
                            nv[i] += nv[j];
                            nv[j] = 0;
                            state[j] = MERGED;
                            merged[i].push_back(j);
                            std::vector<int>().swap(elems[j]);
                            std::vector<int>().swap(vars[j]);
                        }
                    }
                }
            }
            a = b;
        }
        // ---- approximate degrees and the new element's list
        int degme = 0;
        for (int i : keep)
            if (state[i] == VAR) degme += nv[i];
        const int remaining = n - k - nvp;
        auto& Lnew = Le[p];
        Lnew.clear();
        for (int i : keep) {
            if (state[i] != VAR) continue;
            const int ext = degme - nv[i];
            long long d = std::min<long long>((long long)deg[i] + ext, (long long)tmpdeg[i] + ext);
            d = std::min<long long>(d, remaining - nv[i]);
            deg[i] = (int)std::max<long long>(d, 0);
            ins(i);
            mindeg = std::min(mindeg, deg[i]);
            Lnew.push_back(i);
        }
        order.push_back(p);
        k += nvp;
        nv[p] = nvp;
        wflg += (long long)n + 2;
    }
    // expand supervariables / mass-eliminated variables after their pivot
    std::vector<int> perm;
    perm.reserve(n);
    std::vector<int> stack;
    for (int p : order) {
        stack.assign(1, p);
        while (!stack.empty()) {
            const int v = stack.back();
            stack.pop_back();
            perm.push_back(v);
            for (auto it = merged[v].rbegin(); it != merged[v].rend(); ++it) stack.push_back(*it);
        }
    }
    if ((int)perm.size() != n) throw Error{PDGB_ERR_INVALID_ARGUMENT, "internal error: AMD ordering incomplete"};
    return perm;
}

// ------------------------------------------------------ nested dissection
static void nd_rec(std::vector<int>& vs, const SparseSym& A, const float* xyz, std::vector<int>& order,
                   std::vector<int>& mark, int& stamp) {
    if (vs.size() <= 32) {
        order.insert(order.end(), vs.begin(), vs.end());
        return;
    }
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int v : vs)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], xyz[3 * v + d]);
            hi[d] = std::max(hi[d], xyz[3 * v + d]);
        }
    int ax = 0;
    for (int d = 1; d < 3; ++d)
        if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    const size_t half = vs.size() / 2;
    std::nth_element(vs.begin(), vs.begin() + half, vs.end(), [&](int a, int b) {
        const float xa = xyz[3 * a + ax], xb = xyz[3 * b + ax];
        return xa < xb || (xa == xb && a < b);
    });
    const int my = ++stamp;
    for (size_t q = 0; q < half; ++q) mark[vs[q]] = my;
    std::vector<int> Lo(vs.begin(), vs.begin() + half), Hi, Sep;
    for (size_t q = half; q < vs.size(); ++q) {
        const int v = vs[q];
        bool sep = false;
        for (int64_t e = A.p[v]; e < A.p[v + 1] && !sep; ++e) sep = mark[A.i[e]] == my;
        (sep ? Sep : Hi).push_back(v);
    }
    std::vector<int>().swap(vs);
    nd_rec(Lo, A, xyz, order, mark, stamp);
    nd_rec(Hi, A, xyz, order, mark, stamp);
    order.insert(order.end(), Sep.begin(), Sep.end());
}

std::vector<int> nd_order(const SparseSym& A, const float* xyz) {
    std::vector<int> vs(A.n), mark(A.n, 0), order;
    std::iota(vs.begin(), vs.end(), 0);
    order.reserve(A.n);
    int stamp = 0;
    nd_rec(vs, A, xyz, order, mark, stamp);
    return order;
}

// ------------------------------------------------------- symbolic tools
namespace {

// Elimination tree of C = P A P^T (parent[j] > j or -1), Liu's algorithm.
std::vector<int> etree(const SparseSym& A, const std::vector<int>& perm, const std::vector<int>& iperm) {
    const int n = A.n;
    std::vector<int> parent(n, -1), anc(n, -1);
    for (int k = 0; k < n; ++k) {
        const int v = perm[k];
        for (int64_t e = A.p[v]; e < A.p[v + 1]; ++e) {
            int i = iperm[A.i[e]];
            while (i != -1 && i < k) {
                const int nx = anc[i];
                anc[i] = k;
                if (nx == -1) {
                    parent[i] = k;
                    break;
                }
                i = nx;
            }
        }
    }
    return parent;
}

std::vector<int> postorder(const std::vector<int>& parent) {
    const int n = (int)parent.size();
    std::vector<int> head(n, -1), next(n, -1), post;
    post.reserve(n);
    for (int j = n - 1; j >= 0; --j)
        if (parent[j] != -1) {
            next[j] = head[parent[j]];
            head[parent[j]] = j;
        }
    std::vector<int> stack;
    for (int r = 0; r < n; ++r) {
        if (parent[r] != -1) continue;
        stack.push_back(r);
        while (!stack.empty()) {
            const int p = stack.back();
            const int c = head[p];
            if (c == -1) {
                stack.pop_back();
                post.push_back(p);
            } else {
                head[p] = next[c];
                stack.push_back(c);
            }
        }
    }
    return post;
}

// Dense lower-triangular m x m front (column major, leading dimension m):
// factor the first k columns in place (right-looking, blocked).
bool partial_cholesky(double* F, int m, int k) {
    constexpr int NB = 48;
    for (int j0 = 0; j0 < k; j0 += NB) {
        const int j1 = std::min(k, j0 + NB);
        // panel
        for (int j = j0; j < j1; ++j) {
            double* cj = F + (size_t)j * m;
            const double d = cj[j];
            if (!(d > 0.0) || !std::isfinite(d)) return false;
            const double l = std::sqrt(d);
            cj[j] = l;
            const double il = 1.0 / l;
            for (int i = j + 1; i < m; ++i) cj[i] *= il;
            for (int c = j + 1; c < j1; ++c) {
                double* cc = F + (size_t)c * m;
                const double f = cj[c];
                for (int i = c; i < m; ++i) cc[i] -= cj[i] * f;
            }
        }
        // trailing update with the panel: F[c:, c] -= sum_j L[c:, j] L[c, j]
        const int nc = m - j1;
        if (nc <= 0) continue;
#pragma omp parallel for schedule(dynamic, 8) if ((long long)nc * nc * (j1 - j0) > 2000000)
        for (int c = j1; c < m; ++c) {
            double* cc = F + (size_t)c * m;
            for (int j = j0; j < j1; ++j) {
                const double* cj = F + (size_t)j * m;
                const double f = cj[c];
                if (f == 0.0) continue;
                for (int i = c; i < m; ++i) cc[i] -= cj[i] * f;
            }
        }
    }
    return true;
}

}  // namespace

void cholesky_factor(const SparseSym& K, int ordering, const float* xyz, CholFactor& out, int bwd_chunk_rows,
                     bool gpu_numeric, bool finish_plan, int amalgamation) {
    const int n = K.n;
    out = CholFactor();
    out.n = n;
    out.K = K;
    // ---- ordering, then postorder of the elimination tree
    std::vector<int> perm0 = ordering == 1 ? nd_order(K, xyz) : amd_order(K);
    std::vector<int> iperm(n);
    for (int k = 0; k < n; ++k) iperm[perm0[k]] = k;
    {
        std::vector<int> parent = etree(K, perm0, iperm);
        std::vector<int> post = postorder(parent);
        std::vector<int> perm(n);
        for (int k = 0; k < n; ++k) perm[k] = perm0[post[k]];
        perm0.swap(perm);
        for (int k = 0; k < n; ++k) iperm[perm0[k]] = k;
    }
    const std::vector<int>& perm = perm0;
    std::vector<int> parent = etree(K, perm, iperm);
    // ---- column counts via row subtrees (ereach)
    std::vector<int> colcount(n, 1), wmark(n, -1), stk(n);
    for (int k = 0; k < n; ++k) {
        wmark[k] = k;
        const int v = perm[k];
        for (int64_t e = K.p[v]; e < K.p[v + 1]; ++e) {
            int i = iperm[K.i[e]];
            if (i >= k) continue;
            for (; wmark[i] != k; i = parent[i]) {
                wmark[i] = k;
                colcount[i]++;
            }
        }
    }
    long long nnz = 0;
    for (int j = 0; j < n; ++j) nnz += colcount[j];
    out.nnz_L = nnz;
    // ---- fundamental supernodes
    std::vector<int> nchild(n, 0);
    for (int j = 0; j < n; ++j)
        if (parent[j] >= 0) nchild[parent[j]]++;
    std::vector<int> sfirst;  // first column of each supernode
    for (int j = 0; j < n; ++j) {
        const bool cont = j > 0 && parent[j - 1] == j && colcount[j - 1] == colcount[j] + 1 && nchild[j] == 1;
        if (!cont) sfirst.push_back(j);
    }
    // ---- relaxed amalgamation: merge a supernode into its parent when its
    // columns immediately precede the parent's (it is the parent's last child
    // in postorder) and the explicit zeros stay small.  The merged block has
    // the parent's off-diagonal rows, so k = k_s + k_p and m = k_s + m_p.
    // This removes the 1-3 column supernodes that break chains at the top of
    // AMD trees (each one a level of the solve) and most leaf singletons.
    // kAmalgChain: at most 2,048 more zeros, or at most a quarter of the
    // merged block.  The engine's solve is bound by its chain of levels more
    // than by the factor's bytes: against kAmalgBytes (256 zeros or an
    // eighth) this stores 18 % more entries on the 512-body batch and 21 %
    // more on the 40^3 cube, and solves 12 % and 4 % faster (11 levels
    // instead of 14, 14 instead of 16).  kAmalgBytes serves the serving
    // step, whose many requests' solves together are bound by bytes.
    {
        const int nf = (int)sfirst.size();
        sfirst.push_back(n);
        std::vector<long long> bk(nf), bm(nf), btrue(nf);
        for (int s = 0; s < nf; ++s) {
            bk[s] = sfirst[s + 1] - sfirst[s];
            bm[s] = colcount[sfirst[s]];
            long long t = 0;
            for (int j = sfirst[s]; j < sfirst[s + 1]; ++j) t += colcount[j];
            btrue[s] = t;
        }
        std::vector<int> col2f(n);
        for (int s = 0; s < nf; ++s)
            for (int j = sfirst[s]; j < sfirst[s + 1]; ++j) col2f[j] = s;
        // merged[s] = true if block s was merged into the following block
        std::vector<char> merged(nf, 0);
        auto stored = [](long long k, long long m) { return k * m - k * (k - 1) / 2; };
        for (int s = 0; s + 1 < nf; ++s) {
            const int last = sfirst[s + 1] - 1;
            if (parent[last] != sfirst[s + 1]) continue;  // parent block must start right after
            const int p = s + 1;
            const long long k = bk[s] + bk[p], m = bk[s] + bm[p];
            const long long tr = btrue[s] + btrue[p];
            const long long zeros = stored(k, m) - tr;
            const long long added = zeros - (stored(bk[s], bm[s]) - btrue[s]) - (stored(bk[p], bm[p]) - btrue[p]);
            const bool take = amalgamation == kAmalgChain ? (added <= 2048 || zeros * 4 <= stored(k, m))
                                                          : (added <= 256 || zeros * 8 <= stored(k, m));
            if (take) {
                merged[s] = 1;
                bk[p] = k;
                bm[p] = m;
                btrue[p] = tr;
            }
        }
        std::vector<int> sf;
        for (int s = 0; s < nf; ++s)
            if (s == 0 || !merged[s - 1]) sf.push_back(sfirst[s]);
        sfirst.swap(sf);
    }
    if (ordering == 2) sfirst.assign(1, 0);  // one dense supernode: every pivot, every row
    const int ns = (int)sfirst.size();
    sfirst.push_back(n);
    std::vector<int> col2s(n);
    for (int s = 0; s < ns; ++s)
        for (int j = sfirst[s]; j < sfirst[s + 1]; ++j) col2s[j] = s;
    std::vector<int> sparent(ns, -1);
    for (int s = 0; s < ns; ++s) {
        const int last = sfirst[s + 1] - 1;
        if (parent[last] >= 0) sparent[s] = col2s[parent[last]];
    }
    // ---- row structures (symbolic multifrontal), in permuted indices
    std::vector<std::vector<int>> sstruct(ns);
    std::vector<std::vector<int>> schildren(ns);
    for (int s = 0; s < ns; ++s)
        if (sparent[s] >= 0) schildren[sparent[s]].push_back(s);
    std::vector<int> smark(n, -1);
    for (int s = 0; s < ns; ++s) {
        const int f = sfirst[s], l = sfirst[s + 1];
        std::vector<int>& st = sstruct[s];
        for (int j = f; j < l; ++j) {
            st.push_back(j);
            smark[j] = s;
        }
        for (int j = f; j < l; ++j) {
            const int v = perm[j];
            for (int64_t e = K.p[v]; e < K.p[v + 1]; ++e) {
                const int i = iperm[K.i[e]];
                if (i >= l && smark[i] != s) {
                    smark[i] = s;
                    st.push_back(i);
                }
            }
        }
        for (int c : schildren[s])
            for (int i : sstruct[c])
                if (i >= l && smark[i] != s) {
                    smark[i] = s;
                    st.push_back(i);
                }
        std::sort(st.begin() + (l - f), st.end());
        if ((int)st.size() != (l - f) + colcount[l - 1] - 1)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "internal error: supernode structure mismatch"};
    }
    // ---- numeric multifrontal factorisation (FP64) + M_s blocks
    out.nsuper = ns;
    out.sk.resize(ns);
    out.sm.resize(ns);
    out.moff.resize(ns + 1);
    out.roff.resize(ns + 1);
    out.level.assign(ns, 0);
    int64_t mtot = 0, rtot = 0;
    for (int s = 0; s < ns; ++s) {
        out.sk[s] = sfirst[s + 1] - sfirst[s];
        out.sm[s] = (int)sstruct[s].size();
        out.moff[s] = mtot;
        out.roff[s] = (int)rtot;
        mtot += (int64_t)out.sk[s] * out.sm[s];
        rtot += out.sm[s];
    }
    out.moff[ns] = mtot;
    out.roff[ns] = (int)rtot;
    out.mval_size = mtot;
    out.rows.resize(rtot);
    for (int s = 0; s < ns; ++s)
        for (int q = 0; q < out.sm[s]; ++q) out.rows[out.roff[s] + q] = perm[sstruct[s][q]];
    std::vector<int> relpos(n, -1);
    double flops = 0.0;
    if (gpu_numeric) {
        // The numeric factorisation is left to the GPU (factor.cu): record
        // where every entry of K lands in its supernode's front and where
        // every row of a child's Schur complement lands in its parent's.
        FrontPlan& P = out.fp;
        P.on = true;
        P.parent = sparent;
        P.kptr.assign(ns + 1, 0);
        P.rel_ptr.assign(ns + 1, 0);
        for (int s = 0; s < ns; ++s) {
            const int k = out.sk[s], m = out.sm[s], f = sfirst[s];
            if ((int64_t)m * m > (int64_t)INT32_MAX)
                throw Error{PDGB_ERR_UNSUPPORTED, "supernode front too large for the GPU factorisation"};
            const std::vector<int>& st = sstruct[s];
            for (int q = 0; q < m; ++q) relpos[st[q]] = q;
            for (int jj = 0; jj < k; ++jj) {
                const int v = perm[f + jj];
                for (int64_t e = K.p[v]; e < K.p[v + 1]; ++e) {
                    const int i = iperm[K.i[e]];
                    if (i < f + jj) continue;
                    P.kpos.push_back(jj * m + relpos[i]);
                    P.kval.push_back(K.x[e]);
                }
            }
            P.kptr[s + 1] = (int)P.kpos.size();
            for (int jj = 0; jj < k; ++jj) flops += (double)(m - jj) * (m - jj);
            for (int q = 0; q < m; ++q) relpos[st[q]] = -1;
        }
        for (int s = 0; s < ns; ++s) {
            const int p = sparent[s];
            if (p >= 0) {
                const std::vector<int>& sp = sstruct[p];
                for (int q = 0; q < out.sm[p]; ++q) relpos[sp[q]] = q;
                for (int q = out.sk[s]; q < out.sm[s]; ++q) P.rel.push_back(relpos[sstruct[s][q]]);
                for (int q = 0; q < out.sm[p]; ++q) relpos[sp[q]] = -1;
            }
            P.rel_ptr[s + 1] = (int)P.rel.size();
        }
    } else {
        out.mval.assign(mtot, 0.f);
    }
    std::vector<std::vector<double>> upd(ns);  // update matrices (lower, column major)
    std::vector<double> F, Linv;
    for (int s = 0; s < ns && !gpu_numeric; ++s) {
        const int k = out.sk[s], m = out.sm[s], f = sfirst[s];
        const std::vector<int>& st = sstruct[s];
        for (int q = 0; q < m; ++q) relpos[st[q]] = q;
        F.assign((size_t)m * m, 0.0);
        for (int jj = 0; jj < k; ++jj) {
            const int v = perm[f + jj];
            for (int64_t e = K.p[v]; e < K.p[v + 1]; ++e) {
                const int i = iperm[K.i[e]];
                if (i < f + jj) continue;
                F[(size_t)jj * m + relpos[i]] += K.x[e];
            }
        }
        for (int c : schildren[s]) {
            const int kc = out.sk[c], mc = out.sm[c], uc = mc - kc;
            const std::vector<int>& stc = sstruct[c];
            const std::vector<double>& U = upd[c];
            for (int b = 0; b < uc; ++b) {
                const int cb = relpos[stc[kc + b]];
                for (int a = b; a < uc; ++a) F[(size_t)cb * m + relpos[stc[kc + a]]] += U[(size_t)b * uc + a];
            }
            std::vector<double>().swap(upd[c]);
        }
        if (!partial_cholesky(F.data(), m, k))
            throw Error{PDGB_ERR_NOT_SPD, "system matrix is not positive definite (pivot " + std::to_string(f) + ")"};
        for (int jj = 0; jj < k; ++jj) flops += (double)(m - jj) * (m - jj);
        const int u = m - k;
        if (u > 0) {
            upd[s].assign((size_t)u * u, 0.0);
            for (int b = 0; b < u; ++b)
                for (int a = b; a < u; ++a) upd[s][(size_t)b * u + a] = F[(size_t)(k + b) * m + k + a];
        }
        // Linv = L_ss^-1 (k x k lower, column major), column-oriented
        // forward substitution on e_c; then W = L_os Linv by axpys over the
        // contiguous columns of L.
        Linv.assign((size_t)k * k, 0.0);
        float* M = &out.mval[out.moff[s]];
#pragma omp parallel for schedule(dynamic, 4) if ((long long)k * k * m > 4000000)
        for (int c = 0; c < k; ++c) {
            double* x = &Linv[(size_t)c * k];
            x[c] = 1.0;
            for (int q = c; q < k; ++q) {
                const double* Lq = F.data() + (size_t)q * m;
                const double xq = x[q] / Lq[q];
                x[q] = xq;
                if (xq != 0.0)
                    for (int j = q + 1; j < k; ++j) x[j] -= Lq[j] * xq;
            }
            float* Mc = M + (size_t)c * m;
            for (int r = 0; r < k; ++r) Mc[r] = (float)x[r];
            if (m > k) {
                std::vector<double> acc(m - k, 0.0);
                for (int q = c; q < k; ++q) {
                    const double* Lq = F.data() + (size_t)q * m;
                    const double xq = x[q];
                    if (xq == 0.0) continue;
                    for (int r = k; r < m; ++r) acc[r - k] += Lq[r] * xq;
                }
                for (int r = k; r < m; ++r) Mc[r] = (float)acc[r - k];
            }
        }
        for (int q = 0; q < m; ++q) relpos[st[q]] = -1;
    }
    out.flops = flops;
    {
        long long st_tot = 0;
        for (int s = 0; s < ns; ++s) st_tot += (long long)out.sk[s] * out.sm[s] - (long long)out.sk[s] * (out.sk[s] - 1) / 2;
        out.zeros = st_tot - nnz;
    }
    // ---- levels (leaves = 0) and GPU work items
    int nl = 0;
    for (int s = 0; s < ns; ++s) {
        for (int c : schildren[s]) out.level[s] = std::max(out.level[s], out.level[c] + 1);
        nl = std::max(nl, out.level[s] + 1);
    }
    out.nlevels = nl;
    std::vector<std::vector<int>> bylevel(nl);
    for (int s = 0; s < ns; ++s) bylevel[out.level[s]].push_back(s);
    out.levels.resize(nl);
    for (int L = 0; L < nl; ++L) {
        SolveLevel lv;
        lv.fwd_begin = (int)(out.fwd_items.size() / kItemInts);
        lv.bwd_begin = (int)(out.bwd_items.size() / kItemInts);
        lv.fwdb_begin = (int)(out.fwd_blocks.size() / kItemInts);
        lv.bwdb_begin = (int)(out.bwd_blocks.size() / kItemInts);
        lv.fwdw_begin = (int)(out.fwd_small.size() / kItemInts);
        lv.bwdw_begin = (int)(out.bwd_small.size() / kItemInts);
        lv.tiny_begin = (int)(out.tiny.size() / kItemInts);
        lv.zst_begin = (int)(out.zstage.size() / kItemInts);
        for (int s : bylevel[L]) {
            const int k = out.sk[s], m = out.sm[s];
            const int64_t mo = out.moff[s];
            const int lo = (int)(mo & 0xffffffff), hi = (int)(mo >> 32);
            for (int r0 = 0; r0 < m; r0 += kFwdItemRows) {
                // pivot rows only need columns <= row (lower-triangular block)
                const int cmax = std::min(k, r0 + kFwdItemRows);
                for (int c0 = 0; c0 < cmax; c0 += kFwdItemCols)
                    out.fwd_items.insert(out.fwd_items.end(),
                                         {lo, hi, out.roff[s], m, k, r0, c0, std::min(cmax, c0 + kFwdItemCols)});
            }
            for (int c = 0; c < k; ++c) out.bwd_items.insert(out.bwd_items.end(), {lo, hi, out.roff[s], m, k, c, 0, 0});
            if (k <= kTinyCols && m <= kTinyRows) {  // tiny: one thread per supernode (per-level launches)
                out.tiny.insert(out.tiny.end(), {lo, hi, out.roff[s], m, k, 0, 0, 0});
                continue;
            }
            if (m < kBlockMinRows) {  // small: the warp items, again, for the per-level launches
                for (int r0 = 0; r0 < m; r0 += kFwdItemRows) {
                    const int cmax = std::min(k, r0 + kFwdItemRows);
                    for (int c0 = 0; c0 < cmax; c0 += kFwdItemCols)
                        out.fwd_small.insert(out.fwd_small.end(),
                                             {lo, hi, out.roff[s], m, k, r0, c0, std::min(cmax, c0 + kFwdItemCols)});
                }
                for (int c = 0; c < k; ++c) out.bwd_small.insert(out.bwd_small.end(), {lo, hi, out.roff[s], m, k, c, 0, 0});
                continue;
            }
            for (int r0 = 0; r0 < m; r0 += kFwdBlockRows) {
                const int cmax = std::min(k, r0 + kFwdBlockRows);
                for (int c0 = 0; c0 < cmax; c0 += kFwdBlockCols)
                    out.fwd_blocks.insert(out.fwd_blocks.end(),
                                          {lo, hi, out.roff[s], m, k, r0, c0, std::min(cmax, c0 + kFwdBlockCols)});
            }
            const int zoff = (int)out.zrows;
            out.zrows += m;
            const int chunk = bwd_chunk_rows > 0 ? bwd_chunk_rows : m;
            const int split = chunk < m ? 1 : 0;  // columns split into row chunks: x is accumulated
            for (int r0 = 0; r0 < m; r0 += kStageRows)
                out.zstage.insert(out.zstage.end(), {lo, hi, out.roff[s], m, k, r0, split, zoff});
            for (int c0 = 0; c0 < k; c0 += kBwdBlockCols) {
                const int cpack = (int)((unsigned)c0 | ((unsigned)(std::min(k, c0 + kBwdBlockCols) - c0) << kBwdColShift));
                for (int r0 = c0 - c0 % chunk; r0 < m; r0 += chunk)  // rows >= c0 only
                    out.bwd_blocks.insert(out.bwd_blocks.end(),
                                          {lo, hi, out.roff[s], m, r0, cpack, std::min(m, r0 + chunk), zoff});
            }
        }
        lv.fwd_end = (int)(out.fwd_items.size() / kItemInts);
        lv.bwd_end = (int)(out.bwd_items.size() / kItemInts);
        lv.fwdb_end = (int)(out.fwd_blocks.size() / kItemInts);
        lv.bwdb_end = (int)(out.bwd_blocks.size() / kItemInts);
        lv.fwdw_end = (int)(out.fwd_small.size() / kItemInts);
        lv.bwdw_end = (int)(out.bwd_small.size() / kItemInts);
        lv.tiny_end = (int)(out.tiny.size() / kItemInts);
        lv.zst_end = (int)(out.zstage.size() / kItemInts);
        out.levels[L] = lv;
    }
    out.body_level = {0, nl};
    out.body_order = {0};
    out.step_levels = out.levels;
    if (gpu_numeric && finish_plan) finish_front_plan(out);
}

int64_t front_doubles(const CholFactor& f, int s) {
    const int64_t m = f.sm[s], k = f.sk[s];
    return m * m + m * k;
}

void finish_front_plan(CholFactor& out) {
    FrontPlan& P = out.fp;
    const int ns = out.nsuper;
    // children of each supernode, in supernode order
    P.child_ptr.assign(ns + 1, 0);
    for (int s = 0; s < ns; ++s)
        if (P.parent[s] >= 0) P.child_ptr[P.parent[s] + 1]++;
    for (int s = 0; s < ns; ++s) P.child_ptr[s + 1] += P.child_ptr[s];
    P.child.assign(P.child_ptr[ns], 0);
    {
        std::vector<int> fill(P.child_ptr.begin(), P.child_ptr.end() - 1);
        for (int s = 0; s < ns; ++s)
            if (P.parent[s] >= 0) P.child[fill[P.parent[s]]++] = s;
    }
    // supernodes by level (levels from the leaves; a batch's bodies together)
    int nl = 0;
    for (int s = 0; s < ns; ++s) nl = std::max(nl, out.level[s] + 1);
    P.lvl_ptr.assign(nl + 1, 0);
    for (int s = 0; s < ns; ++s) P.lvl_ptr[out.level[s] + 1]++;
    for (int L = 0; L < nl; ++L) P.lvl_ptr[L + 1] += P.lvl_ptr[L];
    P.lvl_sn.assign(ns, 0);
    {
        std::vector<int> fill(P.lvl_ptr.begin(), P.lvl_ptr.end() - 1);
        for (int s = 0; s < ns; ++s) P.lvl_sn[fill[out.level[s]]++] = s;
    }
    // Front pool, best fit: the fronts of level L are placed while their
    // children's fronts still hold the Schur complements they pass up; the
    // children's memory is released once level L is placed.
    P.foff.assign(ns, 0);
    P.max_m = 0;
    std::set<std::pair<int64_t, int64_t>> by_size;  // (size, offset) of the free blocks
    std::map<int64_t, int64_t> by_off;              // offset -> size of a free block
    int64_t top = 0;
    auto take = [&](int64_t need) -> int64_t {
        auto it = by_size.lower_bound({need, INT64_MIN});
        if (it == by_size.end()) {
            const int64_t o = top;
            top += need;
            return o;
        }
        const int64_t size = it->first, o = it->second;
        by_size.erase(it);
        by_off.erase(o);
        if (size > need) {
            by_size.emplace(size - need, o + need);
            by_off.emplace(o + need, size - need);
        }
        return o;
    };
    auto give = [&](int64_t o, int64_t size) {
        auto next = by_off.lower_bound(o);
        if (next != by_off.end() && next->first == o + size) {  // merge with the following block
            by_size.erase({next->second, next->first});
            size += next->second;
            next = by_off.erase(next);
        }
        if (next != by_off.begin()) {  // merge with the preceding block
            auto prev = std::prev(next);
            if (prev->first + prev->second == o) {
                by_size.erase({prev->second, prev->first});
                o = prev->first;
                size += prev->second;
                by_off.erase(prev);
            }
        }
        if (o + size == top) {  // the block ends the pool: shrink it
            top = o;
            return;
        }
        by_off.emplace(o, size);
        by_size.emplace(size, o);
    };
    int64_t peak = 0;
    for (int L = 0; L < nl; ++L) {
        for (int q = P.lvl_ptr[L]; q < P.lvl_ptr[L + 1]; ++q) {
            const int s = P.lvl_sn[q];
            const int64_t m = out.sm[s];
            P.max_m = std::max(P.max_m, (int)m);
            P.foff[s] = take(front_doubles(out, s));
        }
        peak = std::max(peak, top);
        // level L is assembled: its children's fronts are consumed, and its
        // roots need their fronts only during this level
        for (int q = P.lvl_ptr[L]; q < P.lvl_ptr[L + 1]; ++q) {
            const int s = P.lvl_sn[q];
            for (int c = P.child_ptr[s]; c < P.child_ptr[s + 1]; ++c) {
                const int ch = P.child[c];
                give(P.foff[ch], front_doubles(out, ch));
            }
        }
        for (int q = P.lvl_ptr[L]; q < P.lvl_ptr[L + 1]; ++q) {
            const int s = P.lvl_sn[q];
            if (P.parent[s] < 0) give(P.foff[s], front_doubles(out, s));
        }
    }
    P.pool = peak;
}

void cholesky_factor_bodies(int nbodies, const std::vector<int>& vstart, const std::vector<int>& tstart,
                            const uint32_t* tets4, const double* dminv, const double* coef,
                            const std::vector<double>& mdt2, int ordering, const float* xyz, CholFactor& out,
                            bool gpu_numeric) {
    std::vector<CholFactor> fs(nbodies);
    std::vector<int> order(nbodies);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        return tstart[a + 1] - tstart[a] > tstart[b + 1] - tstart[b];
    });
    std::vector<int> failed(nbodies, 0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < nbodies; ++q) {
        const int b = order[q];
        const int v0 = vstart[b], nvb = vstart[b + 1] - v0, t0 = tstart[b], ntb = tstart[b + 1] - t0;
        try {
            std::vector<uint32_t> lt(4 * (size_t)ntb);
            for (size_t i = 0; i < lt.size(); ++i) lt[i] = tets4[4 * (size_t)t0 + i] - (uint32_t)v0;
            std::vector<double> md(mdt2.begin() + v0, mdt2.begin() + v0 + nvb);
            SparseSym Kb = assemble_system(nvb, ntb, lt.data(), dminv + 9 * (size_t)t0, coef + t0, md);
            cholesky_factor(Kb, ordering, xyz ? xyz + 3 * (size_t)v0 : nullptr, fs[b], 0, gpu_numeric, false);
        } catch (const Error& e) {
            failed[b] = e.status;
        } catch (...) {
            failed[b] = PDGB_ERR_OUT_OF_MEMORY;
        }
    }
    for (int b = 0; b < nbodies; ++b)
        if (failed[b])
            throw Error{failed[b], "factorisation of body " + std::to_string(b) + " failed (" +
                                       (failed[b] == PDGB_ERR_NOT_SPD ? "not positive definite" : "error") + ")"};
    out = CholFactor();
    out.n = vstart[nbodies];
    int64_t mbase = 0, rbase = 0, zbase = 0;
    int sbase = 0;
    out.body_level.assign(1, 0);
    // per-level buckets of the block / small items of all bodies
    std::vector<std::vector<int>> bfb, bfw, bbb, bbw, btn, bzs;
    for (int b = 0; b < nbodies; ++b) {
        CholFactor& f = fs[b];
        const int v0 = vstart[b];
        out.nnz_L += f.nnz_L;
        out.zeros += f.zeros;
        out.flops += f.flops;
        out.nlevels = std::max(out.nlevels, f.nlevels);
        for (int s = 0; s < f.nsuper; ++s) {
            out.sk.push_back(f.sk[s]);
            out.sm.push_back(f.sm[s]);
            out.moff.push_back(f.moff[s] + mbase);
            out.roff.push_back(f.roff[s] + (int)rbase);
            out.level.push_back(f.level[s]);
        }
        out.nsuper += f.nsuper;
        out.mval.insert(out.mval.end(), f.mval.begin(), f.mval.end());
        if (gpu_numeric) {
            FrontPlan& P = out.fp;
            const FrontPlan& Q = f.fp;
            if (P.kptr.empty()) {
                P.kptr.assign(1, 0);
                P.rel_ptr.assign(1, 0);
            }
            const int kb = (int)P.kpos.size(), rb = (int)P.rel.size();
            for (int s = 0; s < f.nsuper; ++s) {
                P.parent.push_back(Q.parent[s] >= 0 ? Q.parent[s] + sbase : -1);
                P.kptr.push_back(Q.kptr[s + 1] + kb);
                P.rel_ptr.push_back(Q.rel_ptr[s + 1] + rb);
            }
            P.kpos.insert(P.kpos.end(), Q.kpos.begin(), Q.kpos.end());
            P.kval.insert(P.kval.end(), Q.kval.begin(), Q.kval.end());
            P.rel.insert(P.rel.end(), Q.rel.begin(), Q.rel.end());
        }
        for (int r : f.rows) out.rows.push_back(r + v0);
        auto shift = [&](std::vector<int>& dst, const std::vector<int>& src, bool zfield = false) {
            const int base_item = (int)(dst.size() / kItemInts);
            for (size_t i = 0; i < src.size(); i += kItemInts) {
                const int64_t mo = ((int64_t)(uint32_t)src[i] | ((int64_t)src[i + 1] << 32)) + mbase;
                dst.push_back((int)(mo & 0xffffffff));
                dst.push_back((int)(mo >> 32));
                dst.push_back(src[i + 2] + (int)rbase);
                for (int j = 3; j < kItemInts - 1; ++j) dst.push_back(src[i + j]);
                dst.push_back(src[i + kItemInts - 1] + (zfield ? (int)zbase : 0));
            }
            return base_item;
        };
        const int fb = shift(out.fwd_items, f.fwd_items);
        const int bb = shift(out.bwd_items, f.bwd_items);
        auto slice = [](const std::vector<int>& v, int b0, int b1) {
            return std::vector<int>(v.begin() + (size_t)kItemInts * b0, v.begin() + (size_t)kItemInts * b1);
        };
        if ((int)bfb.size() < f.nlevels) {
            bfb.resize(f.nlevels); bfw.resize(f.nlevels); bbb.resize(f.nlevels); bbw.resize(f.nlevels);
            btn.resize(f.nlevels);
            bzs.resize(f.nlevels);
        }
        for (int L = 0; L < (int)f.levels.size(); ++L) {
            const SolveLevel& lv = f.levels[L];
            out.levels.push_back({lv.fwd_begin + fb, lv.fwd_end + fb, lv.bwd_begin + bb, lv.bwd_end + bb,
                                  0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0});
            shift(btn[L], slice(f.tiny, lv.tiny_begin, lv.tiny_end));
            shift(bzs[L], slice(f.zstage, lv.zst_begin, lv.zst_end), true);
            shift(bfb[L], slice(f.fwd_blocks, lv.fwdb_begin, lv.fwdb_end));
            shift(bfw[L], slice(f.fwd_small, lv.fwdw_begin, lv.fwdw_end));
            shift(bbb[L], slice(f.bwd_blocks, lv.bwdb_begin, lv.bwdb_end), true);
            shift(bbw[L], slice(f.bwd_small, lv.bwdw_begin, lv.bwdw_end));
        }
        out.body_level.push_back((int)out.levels.size());
        mbase += f.mval_size;
        rbase += (int64_t)f.rows.size();
        zbase += f.zrows;
        out.zrows += f.zrows;
        sbase += f.nsuper;
        out.K.n = 0;  // per-body systems are not kept
        f = CholFactor();  // release the per-body copy
    }
    out.mval_size = mbase;
    if (gpu_numeric) {
        out.fp.on = true;
        finish_front_plan(out);
    }
    for (size_t L = 0; L < bfb.size(); ++L) {
        SolveLevel lv{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        auto put = [&](std::vector<int>& dst, std::vector<int>& src, int& b0, int& b1) {
            b0 = (int)(dst.size() / kItemInts);
            dst.insert(dst.end(), src.begin(), src.end());
            b1 = (int)(dst.size() / kItemInts);
            std::vector<int>().swap(src);
        };
        put(out.fwd_blocks, bfb[L], lv.fwdb_begin, lv.fwdb_end);
        put(out.fwd_small, bfw[L], lv.fwdw_begin, lv.fwdw_end);
        put(out.bwd_blocks, bbb[L], lv.bwdb_begin, lv.bwdb_end);
        put(out.bwd_small, bbw[L], lv.bwdw_begin, lv.bwdw_end);
        put(out.tiny, btn[L], lv.tiny_begin, lv.tiny_end);
        put(out.zstage, bzs[L], lv.zst_begin, lv.zst_end);
        out.step_levels.push_back(lv);
    }
    std::vector<std::pair<int64_t, int>> sz(nbodies);
    for (int b = 0; b < nbodies; ++b) {
        int64_t e = 0;
        for (int L = out.body_level[b]; L < out.body_level[b + 1]; ++L)
            e += (int64_t)(out.levels[L].fwd_end - out.levels[L].fwd_begin) + (out.levels[L].bwd_end - out.levels[L].bwd_begin);
        sz[b] = {-e, b};
    }
    std::sort(sz.begin(), sz.end());
    out.body_order.resize(nbodies);
    for (int b = 0; b < nbodies; ++b) out.body_order[b] = sz[b].second;
}

void cholesky_solve_host(const CholFactor& f, const double* b3, double* x3) {
    const int n = f.n;
    std::vector<double> r(b3, b3 + 3 * (size_t)n), y(3 * (size_t)n, 0.0);
    auto moff_of = [](const int* w) { return (int64_t)(uint32_t)w[0] | ((int64_t)w[1] << 32); };
    for (int L = 0; L < (int)f.levels.size(); ++L)
        for (int it = f.levels[L].fwd_begin; it < f.levels[L].fwd_end; ++it) {
            const int* w = &f.fwd_items[kItemInts * (size_t)it];
            const int roff = w[2], m = w[3], k = w[4], r0 = w[5], c0 = w[6], c1 = w[7];
            const float* M = &f.mval[moff_of(w)];
            const int* rows = &f.rows[roff];
            for (int row = r0; row < std::min(m, r0 + kFwdItemRows); ++row) {
                double acc[3] = {0, 0, 0};
                const int cend = row < k ? std::min(c1, row + 1) : c1;
                for (int c = c0; c < cend; ++c)
                    for (int d = 0; d < 3; ++d) acc[d] += (double)M[(size_t)c * m + row] * r[3 * (size_t)rows[c] + d];
                const size_t o = 3 * (size_t)rows[row];
                for (int d = 0; d < 3; ++d) {
                    if (row < k) y[o + d] += acc[d];
                    else r[o + d] -= acc[d];
                }
            }
        }
    // bodies are independent: walk each body's levels top-down
    for (size_t b = 0; b + 1 < f.body_level.size(); ++b)
    for (int L = f.body_level[b + 1] - 1; L >= f.body_level[b]; --L)
        for (int it = f.levels[L].bwd_begin; it < f.levels[L].bwd_end; ++it) {
            const int* w = &f.bwd_items[kItemInts * (size_t)it];
            const int roff = w[2], m = w[3], k = w[4], c = w[5];
            const float* M = &f.mval[moff_of(w)];
            const int* rows = &f.rows[roff];
            double acc[3] = {0, 0, 0};
            for (int i = c; i < m; ++i) {
                const size_t o = 3 * (size_t)rows[i];
                const double mv = M[(size_t)c * m + i];
                for (int d = 0; d < 3; ++d) acc[d] += mv * (i < k ? y[o + d] : -x3[o + d]);
            }
            for (int d = 0; d < 3; ++d) x3[3 * (size_t)rows[c] + d] = acc[d];
        }
}

}  // namespace pdgb

namespace pdgb {

void build_dsm_plan(const CholFactor& f, int ctas, int warps_per_cta, size_t max_smem, DsmPlan& plan) {
    plan = DsmPlan();
    if (f.body_level.size() != 2 || f.nsuper == 0 || ctas < 1) return;  // single bodies only
    const int ns = f.nsuper;
    plan.ctas = ctas;
    plan.n = f.n;
    plan.slots = (f.n + ctas - 1) / ctas;
    plan.nlevels = f.nlevels;
    // supernodes to CTAs: largest M_s first, each to the least loaded CTA
    std::vector<int> order(ns);
    std::iota(order.begin(), order.end(), 0);
    auto msize = [&](int s) { return (int64_t)f.sm[s] * f.sk[s]; };
    std::sort(order.begin(), order.end(), [&](int a, int b) { return msize(a) > msize(b); });
    std::vector<int64_t> load(ctas, 0);
    std::vector<int> owner(ns);
    for (int s : order) {
        const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        owner[s] = c;
        load[c] += msize(s) + f.sm[s];
    }
    // staged areas, per CTA: its supernodes' M_s blocks and row lists back to back
    std::vector<std::vector<int>> mine(ctas);
    for (int s = 0; s < ns; ++s) mine[owner[s]].push_back(s);
    std::vector<int> moff_smem(ns), roff_smem(ns);
    int max_m = 0, max_r = 0;
    plan.mcopy_ptr.assign(1, 0);
    plan.rcopy_ptr.assign(1, 0);
    for (int c = 0; c < ctas; ++c) {
        int mo = 0, ro = 0;
        for (int s : mine[c]) {
            moff_smem[s] = mo;
            const int64_t cnt = (int64_t)f.sm[s] * f.sk[s];
            plan.mcopy.insert(plan.mcopy.end(), f.mval.begin() + f.moff[s], f.mval.begin() + f.moff[s] + cnt);
            mo += (int)cnt;
            roff_smem[s] = ro;
            plan.rcopy.insert(plan.rcopy.end(), f.rows.begin() + f.roff[s], f.rows.begin() + f.roff[s] + f.sm[s]);
            ro += f.sm[s];
        }
        while (plan.mcopy.size() & 3) plan.mcopy.push_back(0.f);
        while (plan.rcopy.size() & 3) plan.rcopy.push_back(0);
        plan.mcopy_ptr.push_back((int)plan.mcopy.size());
        plan.rcopy_ptr.push_back((int)plan.rcopy.size());
        max_m = std::max(max_m, mo);
        max_r = std::max(max_r, ro);
    }
    // shared memory: 3 vectors + warp staging (float4), M, rows
    const int vec_f4 = 3 * plan.slots + warps_per_cta * 32;
    plan.m_area = 4 * vec_f4;
    plan.r_area = plan.m_area + ((max_m + 3) & ~3);
    plan.smem_bytes = 4 * (size_t)plan.r_area + 4 * (size_t)((max_r + 3) & ~3);
    if (plan.smem_bytes > max_smem) return;
    // items per CTA and level
    std::vector<std::vector<int>> bylevel(f.nlevels);
    for (int s = 0; s < ns; ++s) bylevel[f.level[s]].push_back(s);
    plan.lvl.assign((size_t)ctas * f.nlevels * 4, 0);
    for (int c = 0; c < ctas; ++c)
        for (int L = 0; L < f.nlevels; ++L) {
            int* lv = &plan.lvl[((size_t)c * f.nlevels + L) * 4];
            lv[0] = (int)(plan.items.size() / kItemInts);
            for (int s : bylevel[L]) {
                if (owner[s] != c) continue;
                const int k = f.sk[s], m = f.sm[s];
                for (int r0 = 0; r0 < m; r0 += kFwdItemRows) {
                    const int cmax = std::min(k, r0 + kFwdItemRows);
                    for (int c0 = 0; c0 < cmax; c0 += kFwdItemCols)
                        plan.items.insert(plan.items.end(), {moff_smem[s], roff_smem[s], m, k, r0, c0,
                                                             std::min(cmax, c0 + kFwdItemCols), 0});
                }
            }
            lv[1] = (int)(plan.items.size() / kItemInts);
            lv[2] = lv[1];
            for (int s : bylevel[L]) {
                if (owner[s] != c) continue;
                for (int col = 0; col < f.sk[s]; ++col)
                    plan.items.insert(plan.items.end(), {moff_smem[s], roff_smem[s], f.sm[s], f.sk[s], col, 0, 0, 0});
            }
            lv[3] = (int)(plan.items.size() / kItemInts);
        }
    plan.ok = true;
}

}  // namespace pdgb
