// setup.cpp -- host-side integer set-up of the Schwarz preconditioners:
// decomposition (src/decomp/domain_decomp.h:61-93), owned-local map
// (src/precond/ras.h:34-41), local CSR structure of A[dofs,dofs]
// (src/core/sparse_matrix.h:53-83), ILU(0) diagonal positions
// (src/precond/ilu0.h:19-29) and the level schedules of the two sweeps.
// All of it is integer work; the floating-point set-up (value gather,
// factorisation, coarse operator) runs on the device (schwarz.cu).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <exception>
#include <mutex>
#include <numeric>
#include <thread>

#include "sg_internal.h"

namespace sg {

void schwarz_finish(sg_precond* pc, const std::vector<int>& perm_f_all,
                    const std::vector<int>& perm_b_all);

// Level of every row of one local CSR for the forward sweep (reads columns
// before the first column >= row, src/precond/ilu0.h:62-67) and for the
// backward sweep (reads the entries after the diagonal, :70-76).
static int levels_lower(int n, const int* rp, const int* ci, int* lev) {
    int nlev = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int e = rp[i]; e < rp[i + 1]; ++e) {
            const int c = ci[e];
            if (c >= i) break;
            l = std::max(l, lev[c] + 1);
        }
        lev[i] = l;
        nlev = std::max(nlev, l + 1);
    }
    return nlev;
}

static int levels_upper(int n, const int* rp, const int* ci, const int* dg, int* lev) {
    int nlev = 0;
    for (int i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int e = dg[i] + 1; e < rp[i + 1]; ++e) l = std::max(l, lev[ci[e]] + 1);
        lev[i] = l;
        nlev = std::max(nlev, l + 1);
    }
    return nlev;
}

// rows sorted by level (stable): perm[p] = row, ptr[l] = first position of level l
// Bank-conflict cost of the TMA sweep's loads of the subdomain vector t under
// the slot layout tslot(., p): per level, each warp (32 consecutive rows)
// loads t[r] and t[c_k] for k < w (padding columns read t[n]); a load costs
// the largest number of distinct slots that share a bank (4-byte banks,
// `words` banks per element).  Sums over both sweeps.
static long long sweep_bank_cost(int n, const int* lrp, const int* lci, const int* ldg,
                                 const int* perm_f, const int* ptr_f, int nlf,
                                 const int* perm_b, const int* ptr_b, int nlb, int wl, int wu,
                                 int p, int words) {
    long long cost = 0;
    int slots[32], cnt[32];
    auto load_cost = [&](int m) {
        // distinct slots per bank group
        std::sort(slots, slots + m);
        for (int b = 0; b < 32; ++b) cnt[b] = 0;
        int mx = 0;
        for (int i = 0; i < m; ++i) {
            if (i > 0 && slots[i] == slots[i - 1]) continue;
            const int b = (int)(((long long)slots[i] * words) % 32) / words;
            mx = std::max(mx, ++cnt[b]);
        }
        return mx;
    };
    for (int pass = 0; pass < 2; ++pass) {
        const int* perm = pass ? perm_b : perm_f;
        const int* ptr = pass ? ptr_b : ptr_f;
        const int nl = pass ? nlb : nlf, w = pass ? wu : wl;
        for (int l = 0; l < nl; ++l) {
            for (int q0 = ptr[l]; q0 < ptr[l + 1]; q0 += 32) {
                const int m = std::min(32, ptr[l + 1] - q0);
                for (int i = 0; i < m; ++i) slots[i] = tslot(perm[q0 + i], p);
                cost += load_cost(m);
                for (int k = 0; k < w; ++k) {
                    for (int i = 0; i < m; ++i) {
                        const int r = perm[q0 + i];
                        int col = n;
                        if (pass == 0) {
                            const int e = lrp[r] + k;
                            if (e < lrp[r + 1] && lci[e] < r) col = lci[e];
                        } else {
                            const int e = ldg[r] + 1 + k;
                            if (e < lrp[r + 1]) col = lci[e];
                        }
                        slots[i] = tslot(col, p);
                    }
                    cost += load_cost(m);
                }
            }
        }
    }
    return cost;
}

// Host threads for the per-subdomain set-up: the hardware threads, at most
// 32 and at most one per subdomain.
static int host_threads(int nparts) {
    unsigned hw = std::thread::hardware_concurrency();
    int t = hw == 0 ? 4 : (int)hw;
    t = std::min(t, 32);
    return std::max(1, std::min(t, nparts));
}

// f(s, scratch) for s in [0, count): subdomains dealt out dynamically to
// `threads` threads; each thread keeps one scratch vector across its calls.
// The first exception thrown by a call is rethrown after all threads end.
template <class F>
static void parallel_for(int count, int threads, F&& f) {
    std::atomic<int> next{0};
    std::exception_ptr err;
    std::mutex err_mu;
    auto work = [&] {
        std::vector<int> scratch;
        for (;;) {
            const int s = next.fetch_add(1);
            if (s >= count) return;
            try {
                f(s, scratch);
            } catch (...) {
                std::lock_guard<std::mutex> lk(err_mu);
                if (!err) err = std::current_exception();
                next.store(count);
                return;
            }
        }
    };
    if (threads <= 1) {
        work();
    } else {
        std::vector<std::thread> pool;
        pool.reserve(threads - 1);
        for (int i = 0; i < threads - 1; ++i) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
    }
    if (err) std::rethrow_exception(err);
}

static void level_order(int n, const int* lev, int nlev, std::vector<int>& perm,
                        std::vector<int>& ptr) {
    ptr.assign(nlev + 1, 0);
    for (int i = 0; i < n; ++i) ptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    perm.resize(n);
    for (int i = 0; i < n; ++i) perm[fill[lev[i]]++] = i;
}

void build_schwarz_host(sg_precond* pc, const sg_csr* A, const int* part_in, int nparts,
                        int overlap) {
    const int n = A->nrows;
    const int* rp = A->h_rp.data();
    const int* ci = A->h_ci.data();
    SG_CHECK_ARG(nparts >= 1, "nparts must be >= 1 (got %d)", nparts);
    SG_CHECK_ARG(overlap >= 0, "overlap must be >= 0 (got %d)", overlap);
    SG_CHECK_ARG(A->nrows == A->ncols, "Schwarz/ILU preconditioners need a square matrix");
    SG_CHECK_ARG(A->sorted, "ILU(0) needs column indices sorted within each row");
    pc->nparts = nparts;
    pc->part.assign(part_in, part_in + n);
    for (int i = 0; i < n; ++i)
        SG_CHECK_ARG(pc->part[i] >= 0 && pc->part[i] < nparts,
                     "partition[%d] = %d is outside [0,%d)", i, pc->part[i], nparts);

    // owned_dofs[s], ascending (src/decomp/domain_decomp.h:64-66)
    pc->owned_ptr.assign(nparts + 1, 0);
    for (int i = 0; i < n; ++i) pc->owned_ptr[pc->part[i] + 1]++;
    for (int s = 0; s < nparts; ++s) pc->owned_ptr[s + 1] += pc->owned_ptr[s];
    pc->owned.resize(n);
    {
        std::vector<int> fill(pc->owned_ptr.begin(), pc->owned_ptr.end() - 1);
        for (int i = 0; i < n; ++i) pc->owned[fill[pc->part[i]]++] = i;
    }
    for (int s = 0; s < nparts; ++s)
        if (pc->owned_ptr[s + 1] == pc->owned_ptr[s])
            fail(SG_ERR_INVALID_ARG, "subdomain %d owns no rows", s);

    // The per-subdomain work below is independent across subdomains: it runs
    // on host threads (each with its own scratch), every subdomain writes its
    // results to its own slots, and the concatenation afterwards keeps the
    // subdomain order -- the output is the same for any thread count.
    const int nthreads = host_threads(nparts);

    // overlap: vertices within `overlap` hops of the owned set, sorted
    // (src/decomp/domain_decomp.h:68-90); owned-local map (ras.h:34-41)
    std::vector<std::vector<int>> sub_s(nparts), ownloc_s(nparts);
    parallel_for(nparts, nthreads, [&](int s, std::vector<int>& scratch) {
        // scratch: a mark array over the global rows, 0 between subdomains
        if (scratch.size() != (size_t)n) scratch.assign(n, 0);
        int* mark = scratch.data();
        std::vector<int>& set = sub_s[s];
        set.assign(pc->owned.begin() + pc->owned_ptr[s], pc->owned.begin() + pc->owned_ptr[s + 1]);
        for (int v : set) mark[v] = 1;
        size_t lo = 0;
        for (int layer = 0; layer < overlap; ++layer) {
            const size_t hi = set.size();
            for (size_t q = lo; q < hi; ++q) {
                const int r = set[q];
                for (int e = rp[r]; e < rp[r + 1]; ++e) {
                    const int c = ci[e];
                    if (!mark[c]) {
                        mark[c] = 1;
                        set.push_back(c);
                    }
                }
            }
            lo = hi;
        }
        std::sort(set.begin(), set.end());
        std::vector<int>& ol = ownloc_s[s];
        for (size_t q = 0; q < set.size(); ++q) {
            mark[set[q]] = 0;
            if (pc->part[set[q]] == s) ol.push_back((int)q);
        }
    });
    pc->sub_ptr.assign(nparts + 1, 0);
    pc->ownloc_ptr.assign(nparts + 1, 0);
    for (int s = 0; s < nparts; ++s) {
        pc->sub_ptr[s + 1] = pc->sub_ptr[s] + (int)sub_s[s].size();
        pc->ownloc_ptr[s + 1] = pc->ownloc_ptr[s] + (int)ownloc_s[s].size();
    }
    pc->sub.resize(pc->sub_ptr[nparts]);
    pc->ownloc.resize(pc->ownloc_ptr[nparts]);
    for (int s = 0; s < nparts; ++s) {
        std::copy(sub_s[s].begin(), sub_s[s].end(), pc->sub.begin() + pc->sub_ptr[s]);
        std::copy(ownloc_s[s].begin(), ownloc_s[s].end(), pc->ownloc.begin() + pc->ownloc_ptr[s]);
        std::vector<int>().swap(sub_s[s]);
        std::vector<int>().swap(ownloc_s[s]);
    }

    // local CSR A[dofs,dofs] in row order, entries in original order
    // (src/core/sparse_matrix.h:53-83), the global entry of each local one,
    // ILU(0) diagonal positions, widths, level schedules and the slot layout
    const size_t nsub = pc->sub.size();
    pc->ldiag.assign(nsub, -1);
    pc->lev_lo.assign(nsub, 0);
    pc->lev_up.assign(nsub, 0);
    pc->h_info.assign(nparts, SubInfo{});
    std::vector<int> perm_f_all(nsub), perm_b_all(nsub);
    struct LocalOut {
        std::vector<int> lrp, lci, lmap, ptr_f, ptr_b;
        int missing_diag = -1;  // global row without a diagonal entry (-1: none)
    };
    std::vector<LocalOut> lo_s(nparts);
    parallel_for(nparts, nthreads, [&](int s, std::vector<int>& scratch) {
        // scratch: global row -> local row (-1 outside the subdomain)
        if (scratch.size() != (size_t)n) scratch.assign(n, -1);
        int* loc = scratch.data();
        LocalOut& L = lo_s[s];
        const int off = pc->sub_ptr[s];
        const int ns = pc->sub_ptr[s + 1] - off;
        const int* dofs = pc->sub.data() + off;
        for (int li = 0; li < ns; ++li) loc[dofs[li]] = li;
        SubInfo& inf = pc->h_info[s];
        inf.n = ns;
        inf.row_off = off;
        L.lrp.reserve((size_t)ns + 1);
        for (int li = 0; li < ns; ++li) {
            const int gi = dofs[li];
            L.lrp.push_back((int)L.lci.size());
            for (int e = rp[gi]; e < rp[gi + 1]; ++e) {
                const int lj = loc[ci[e]];
                if (lj >= 0) {
                    if (lj == li && pc->ldiag[off + li] < 0)
                        pc->ldiag[off + li] = (int)L.lci.size();
                    L.lci.push_back(lj);
                    L.lmap.push_back(e);
                }
            }
        }
        L.lrp.push_back((int)L.lci.size());
        for (int li = 0; li < ns; ++li) loc[dofs[li]] = -1;
        const int* lrp = L.lrp.data();
        const int* lci = L.lci.data();
        for (int li = 0; li < ns; ++li)
            if (pc->ldiag[off + li] < 0) {
                L.missing_diag = dofs[li];
                return;
            }
        // widths
        int wl = 0, wu = 0;
        for (int li = 0; li < ns; ++li) {
            int cl = 0;
            for (int e = lrp[li]; e < lrp[li + 1] && lci[e] < li; ++e) ++cl;
            wl = std::max(wl, cl);
            wu = std::max(wu, lrp[li + 1] - (pc->ldiag[off + li] + 1));
        }
        inf.wl = wl;
        inf.wu = wu;
        // level schedules
        int* lo = pc->lev_lo.data() + off;
        int* up = pc->lev_up.data() + off;
        const int nlf = levels_lower(ns, lrp, lci, lo);
        const int nlb = levels_upper(ns, lrp, lci, pc->ldiag.data() + off, up);
        inf.nlev_f = nlf;
        inf.nlev_b = nlb;
        std::vector<int> perm;
        level_order(ns, lo, nlf, perm, L.ptr_f);
        std::copy(perm.begin(), perm.end(), perm_f_all.begin() + off);
        level_order(ns, up, nlb, perm, L.ptr_b);
        std::copy(perm.begin(), perm.end(), perm_b_all.begin() + off);
        // slot layout of the TMA-fed sweep: the cheapest of none / one pad
        // word per 32 / per 16 rows under the bank model (slots stay 16-bit)
        {
            const int words = pc->opts.sweep_dtype == SG_FP64 ? 2 : 1;
            const int* dgl = pc->ldiag.data() + off;
            const int* pf = perm_f_all.data() + off;
            inf.tshift = 0;
            long long best = -1;
            for (int p : {0, 5, 4}) {
                if (tslot(ns, p) > 65535) continue;
                const long long c = sweep_bank_cost(ns, lrp, lci, dgl, pf, L.ptr_f.data(), nlf,
                                                    perm.data(), L.ptr_b.data(), nlb, wl, wu, p,
                                                    words);
                if (best < 0 || c < best) {
                    best = c;
                    inf.tshift = p;
                }
            }
        }
        inf.n_own = pc->ownloc_ptr[s + 1] - pc->ownloc_ptr[s];
        inf.own_off = pc->ownloc_ptr[s];
        inf.cscale = 1.0 / std::sqrt((double)(pc->owned_ptr[s + 1] - pc->owned_ptr[s]));
    });
    for (int s = 0; s < nparts; ++s)
        if (lo_s[s].missing_diag >= 0)
            fail(SG_ERR_SINGULAR, "ILU(0): row %d has no diagonal entry", lo_s[s].missing_diag);
    // concatenation in subdomain order
    pc->lrp.clear();
    pc->lci.clear();
    pc->lmap.clear();
    pc->h_lev_ptr_f.clear();
    pc->h_lev_ptr_b.clear();
    {
        size_t nr = 0, nz = 0;
        for (const auto& L : lo_s) {
            nr += L.lrp.size();
            nz += L.lci.size();
        }
        pc->lrp.reserve(nr);
        pc->lci.reserve(nz);
        pc->lmap.reserve(nz);
    }
    for (int s = 0; s < nparts; ++s) {
        LocalOut& L = lo_s[s];
        SubInfo& inf = pc->h_info[s];
        inf.csr_row_off = (int)pc->lrp.size();
        inf.csr_nz_off = (long long)pc->lci.size();
        pc->lrp.insert(pc->lrp.end(), L.lrp.begin(), L.lrp.end());
        pc->lci.insert(pc->lci.end(), L.lci.begin(), L.lci.end());
        pc->lmap.insert(pc->lmap.end(), L.lmap.begin(), L.lmap.end());
        inf.lev_off_f = (int)pc->h_lev_ptr_f.size();
        pc->h_lev_ptr_f.insert(pc->h_lev_ptr_f.end(), L.ptr_f.begin(), L.ptr_f.end());
        inf.lev_off_b = (int)pc->h_lev_ptr_b.size();
        pc->h_lev_ptr_b.insert(pc->h_lev_ptr_b.end(), L.ptr_b.begin(), L.ptr_b.end());
        L = LocalOut();  // release as we go
    }
    schwarz_finish(pc, perm_f_all, perm_b_all);
}

// What both set-up paths (host threads, or the device kernels of
// setup_gpu.cu) finish on the host once every subdomain's local structure,
// level schedules and slot layout are in pc (concatenated in subdomain
// order) and perm_f_all / perm_b_all hold the level orders: factor offsets,
// vector sizes, 16-bit level orders, the level records' layout and the
// launch order.
void schwarz_finish(sg_precond* pc, const std::vector<int>& perm_f_all,
                    const std::vector<int>& perm_b_all) {
    const int nparts = pc->nparts;
    long long fl_total = 0, fu_total = 0;
    int max_n = 0, t_len = 0;
    for (int s = 0; s < nparts; ++s) {
        SubInfo& inf = pc->h_info[s];
        t_len = std::max(t_len, tslot(inf.n, inf.tshift) + 1);
        inf.fl_off = fl_total;
        inf.fu_off = fu_total;
        fl_total += (long long)inf.wl * inf.n;
        fu_total += (long long)inf.wu * inf.n;
        max_n = std::max(max_n, inf.n);
    }
    pc->fl_total = fl_total > 0 ? fl_total : 1;
    pc->fu_total = fu_total > 0 ? fu_total : 1;
    pc->max_n = max_n;
    pc->t_len = t_len;
    pc->total_rows = (long long)pc->sub.size();
    pc->wide_cols = max_n > 65534;
    if (pc->wide_cols) {
        pc->h_perm_f32 = perm_f_all;
        pc->h_perm_b32 = perm_b_all;
    } else {
        pc->h_perm_f16.assign(perm_f_all.begin(), perm_f_all.end());
        pc->h_perm_b16.assign(perm_b_all.begin(), perm_b_all.end());
    }
    const size_t elt = pc->opts.sweep_dtype == SG_FP64 ? 8 : 4;
    pc->use_smem = (size_t)(max_n + 1) * elt <= 220u * 1024u;
    // level records (TMA-fed sweep): rows padded to a multiple of 8 so every
    // segment of a record (2-byte rows/columns, 2/4/8-byte values) is a
    // multiple of 16 bytes and every record starts 16-byte aligned
    {
        const long long sf = pc->opts.sweep_dtype == SG_FP64 ? 8
                             : (pc->opts.factor_dtype == SG_BF16 ? 2 : 4);
        pc->h_rec_off_f.assign(pc->h_lev_ptr_f.size(), 0);
        pc->h_rec_off_b.assign(pc->h_lev_ptr_b.size(), 0);
        pc->h_rec_rows_f.assign(pc->h_lev_ptr_f.size(), 0);
        pc->h_rec_rows_b.assign(pc->h_lev_ptr_b.size(), 0);
        long long cur = 0, mx = 0;
        for (int s = 0; s < nparts; ++s) {
            const SubInfo& inf = pc->h_info[s];
            for (int l = 0; l < inf.nlev_f; ++l) {
                const int c = pc->h_lev_ptr_f[inf.lev_off_f + l + 1] - pc->h_lev_ptr_f[inf.lev_off_f + l];
                const int cp = (c + 7) & ~7;
                const long long bytes = (long long)cp * (2 + inf.wl * (2 + sf));
                pc->h_rec_off_f[inf.lev_off_f + l] = cur;
                pc->h_rec_rows_f[inf.lev_off_f + l] = cp;
                cur += bytes;
                mx = std::max(mx, bytes);
            }
            for (int l = 0; l < inf.nlev_b; ++l) {
                const int c = pc->h_lev_ptr_b[inf.lev_off_b + l + 1] - pc->h_lev_ptr_b[inf.lev_off_b + l];
                const int cp = (c + 7) & ~7;
                const long long bytes = (long long)cp * (2 + inf.wu * (2 + sf) + sf);
                pc->h_rec_off_b[inf.lev_off_b + l] = cur;
                pc->h_rec_rows_b[inf.lev_off_b + l] = cp;
                cur += bytes;
                mx = std::max(mx, bytes);
            }
        }
        pc->rec_total = cur;
        pc->max_levels = 0;
        for (int s2 = 0; s2 < nparts; ++s2)
            pc->max_levels = std::max(pc->max_levels, pc->h_info[s2].nlev_f + pc->h_info[s2].nlev_b);
        pc->rec_stage_bytes = mx;
        pc->use_rec = !pc->wide_cols && pc->use_smem && mx > 0;
    }
    pc->h_cscale.resize(nparts);
    for (int s = 0; s < nparts; ++s) pc->h_cscale[s] = pc->h_info[s].cscale;
    // launch order: largest subdomains first
    pc->h_order.resize(nparts);
    std::iota(pc->h_order.begin(), pc->h_order.end(), 0);
    std::stable_sort(pc->h_order.begin(), pc->h_order.end(), [&](int a, int b) {
        const long long ca = (long long)pc->h_info[a].n * (pc->h_info[a].nlev_f + pc->h_info[a].nlev_b);
        const long long cb = (long long)pc->h_info[b].n * (pc->h_info[b].nlev_f + pc->h_info[b].nlev_b);
        return ca > cb;
    });
}

// ---------------------------------------------------------------- partitioners
// Recursive bisection by breadth-first level structure: each group of
// vertices is ordered by BFS from a pseudo-peripheral vertex (two sweeps,
// ties by lowest index) and cut at the size proportional to the parts asked
// of each half.  Deterministic; disconnected groups continue from their
// lowest unvisited vertex.
void partition_graph(int n, const int* rp, const int* ci, int nparts, int* part) {
    SG_CHECK_ARG(n >= 0 && nparts >= 1, "bad partition arguments");
    if (nparts == 1 || n == 0) {
        std::fill(part, part + n, 0);
        return;
    }
    SG_CHECK_ARG(nparts <= n, "nparts (%d) exceeds the number of rows (%d)", nparts, n);
    std::vector<int> group(n, 0);  // group id of each vertex during recursion
    std::vector<int> visit(n, -1);
    int stamp = 0;
    struct Task {
        std::vector<int> verts;  // ascending
        int k, base, gid;
    };
    std::vector<Task> stack;
    std::vector<int> all(n);
    std::iota(all.begin(), all.end(), 0);
    stack.push_back({std::move(all), nparts, 0, 0});
    int next_gid = 1;
    std::vector<int> order, queue;
    auto bfs = [&](const std::vector<int>& verts, int gid, int start, std::vector<int>& out) {
        // BFS restricted to group gid; continues over components in index order
        ++stamp;
        out.clear();
        size_t scan = 0;
        int src = start;
        while (true) {
            if (visit[src] != stamp) {
                visit[src] = stamp;
                size_t head = out.size();
                out.push_back(src);
                while (head < out.size()) {
                    const int v = out[head++];
                    for (int e = rp[v]; e < rp[v + 1]; ++e) {
                        const int c = ci[e];
                        if (c >= 0 && c < n && group[c] == gid && visit[c] != stamp) {
                            visit[c] = stamp;
                            out.push_back(c);
                        }
                    }
                }
            }
            while (scan < verts.size() && visit[verts[scan]] == stamp) ++scan;
            if (scan >= verts.size()) break;
            src = verts[scan];
        }
    };
    while (!stack.empty()) {
        Task t = std::move(stack.back());
        stack.pop_back();
        if (t.k == 1) {
            for (int v : t.verts) part[v] = t.base;
            continue;
        }
        const int k1 = t.k / 2, k2 = t.k - k1;
        bfs(t.verts, t.gid, t.verts.front(), order);
        bfs(t.verts, t.gid, order.back(), order);
        const size_t cut = (size_t)((long long)t.verts.size() * k1 / t.k);
        const int g1 = next_gid++, g2 = next_gid++;
        std::vector<int> a(order.begin(), order.begin() + cut), b(order.begin() + cut, order.end());
        for (int v : a) group[v] = g1;
        for (int v : b) group[v] = g2;
        std::sort(a.begin(), a.end());
        std::sort(b.begin(), b.end());
        stack.push_back({std::move(b), k2, t.base + k1, g2});
        stack.push_back({std::move(a), k1, t.base, g1});
    }
}

static inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline double u01(uint64_t& s) { return (double)(splitmix64(s) >> 11) * 0x1.0p-53; }

// Recursive coordinate bisection of a grid into boxes with seeded uneven cuts.
void partition_boxes(int nx, int ny, int nz, int nparts, double spread, uint64_t seed,
                     int* part) {
    SG_CHECK_ARG(nx > 0 && ny > 0 && nz > 0 && nparts >= 1, "bad box partition arguments");
    SG_CHECK_ARG(spread >= 0.0 && spread < 0.5, "spread must be in [0,0.5)");
    uint64_t rng = seed;
    struct Box {
        int x0, x1, y0, y1, z0, z1, k, base;
    };
    std::vector<Box> stack{{0, nx, 0, ny, 0, nz, nparts, 0}};
    while (!stack.empty()) {
        Box b = stack.back();
        stack.pop_back();
        if (b.k == 1) {
            for (int z = b.z0; z < b.z1; ++z)
                for (int y = b.y0; y < b.y1; ++y)
                    for (int x = b.x0; x < b.x1; ++x) part[((size_t)z * ny + y) * nx + x] = b.base;
            continue;
        }
        const int k1 = b.k / 2, k2 = b.k - k1;
        const int ex = b.x1 - b.x0, ey = b.y1 - b.y0, ez = b.z1 - b.z0;
        int axis = 0, len = ex;
        if (ey > len) { axis = 1; len = ey; }
        if (ez > len) { axis = 2; len = ez; }
        SG_CHECK_ARG(len >= 2, "grid too small for %d parts", nparts);
        const double f = (double)k1 / b.k * (1.0 + spread * (2.0 * u01(rng) - 1.0));
        int cut = (int)std::lround(f * len);
        cut = std::max(1, std::min(len - 1, cut));
        Box a = b, c = b;
        a.k = k1;
        c.k = k2;
        c.base = b.base + k1;
        if (axis == 0) { a.x1 = b.x0 + cut; c.x0 = b.x0 + cut; }
        else if (axis == 1) { a.y1 = b.y0 + cut; c.y0 = b.y0 + cut; }
        else { a.z1 = b.z0 + cut; c.z0 = b.z0 + cut; }
        stack.push_back(c);
        stack.push_back(a);
    }
}

// ---------------------------------------------------------------- generators
// make_poisson_2d / make_poisson_3d (src/mesh/poisson.h:10-74)
int gen_poisson2d(int nx, int ny, int* rp, int* ci, double* v) {
    int nz = 0;
    auto put = [&](int c, double val) {
        if (ci) { ci[nz] = c; v[nz] = val; }
        ++nz;
    };
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            const int idx = iy * nx + ix;
            if (rp) rp[idx] = nz;
            if (iy > 0) put(idx - nx, -1.0);
            if (ix > 0) put(idx - 1, -1.0);
            put(idx, 4.0);
            if (ix < nx - 1) put(idx + 1, -1.0);
            if (iy < ny - 1) put(idx + nx, -1.0);
        }
    if (rp) rp[nx * ny] = nz;
    return nz;
}

// -div(K grad u) on an nx*ny grid with the constant anisotropic tensor
// K = R(theta) diag(1, eps) R(theta)^T, unit mesh width, Dirichlet boundary
// (neighbours outside the grid dropped).  9-point stencil: second
// differences along x and y, the central difference
// u_xy ~ (u_NE - u_NW - u_SE + u_SW) / 4 for the cross term, so
//   centre 2 Kxx + 2 Kyy, W/E -Kxx, S/N -Kyy, SW/NE -Kxy/2, SE/NW +Kxy/2.
// Row index iy*nx + ix; entries in ascending column order.
int gen_aniso2d(int nx, int ny, double eps, double theta, int* rp, int* ci, double* v) {
    const double c = std::cos(theta), s = std::sin(theta);
    const double kxx = c * c + eps * s * s;
    const double kyy = s * s + eps * c * c;
    const double kxy = (1.0 - eps) * s * c;
    int nz = 0;
    auto put = [&](int col, double val) {
        if (ci) { ci[nz] = col; v[nz] = val; }
        ++nz;
    };
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            const int idx = iy * nx + ix;
            if (rp) rp[idx] = nz;
            if (iy > 0) {
                if (ix > 0) put(idx - nx - 1, -0.5 * kxy);
                put(idx - nx, -kyy);
                if (ix < nx - 1) put(idx - nx + 1, 0.5 * kxy);
            }
            if (ix > 0) put(idx - 1, -kxx);
            put(idx, 2.0 * kxx + 2.0 * kyy);
            if (ix < nx - 1) put(idx + 1, -kxx);
            if (iy < ny - 1) {
                if (ix > 0) put(idx + nx - 1, 0.5 * kxy);
                put(idx + nx, -kyy);
                if (ix < nx - 1) put(idx + nx + 1, -0.5 * kxy);
            }
        }
    if (rp) rp[nx * ny] = nz;
    return nz;
}

// 7-point operator with per-face coefficients; k == 1 gives make_poisson_3d
static int gen_faces3d(int nx, int ny, int nz_, const double* kc, int* rp, int* ci, double* v) {
    const int nxy = nx * ny;
    int nz = 0;
    auto put = [&](int c, double val) {
        if (ci) { ci[nz] = c; v[nz] = val; }
        ++nz;
    };
    auto face = [&](int a, int b) {
        if (!kc) return 1.0;
        return 2.0 * kc[a] * kc[b] / (kc[a] + kc[b]);
    };
    for (int iz = 0; iz < nz_; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const int idx = iz * nxy + iy * nx + ix;
                if (rp) rp[idx] = nz;
                const double kself = kc ? kc[idx] : 1.0;
                double diag = 0.0;
                // the six faces; a face on the boundary couples to the
                // Dirichlet value 0 with the cell's own coefficient
                const double fzm = iz > 0 ? face(idx, idx - nxy) : kself;
                const double fym = iy > 0 ? face(idx, idx - nx) : kself;
                const double fxm = ix > 0 ? face(idx, idx - 1) : kself;
                const double fxp = ix < nx - 1 ? face(idx, idx + 1) : kself;
                const double fyp = iy < ny - 1 ? face(idx, idx + nx) : kself;
                const double fzp = iz < nz_ - 1 ? face(idx, idx + nxy) : kself;
                diag = fzm + fym + fxm + fxp + fyp + fzp;
                if (!kc) diag = 6.0;
                if (iz > 0) put(idx - nxy, -fzm);
                if (iy > 0) put(idx - nx, -fym);
                if (ix > 0) put(idx - 1, -fxm);
                put(idx, diag);
                if (ix < nx - 1) put(idx + 1, -fxp);
                if (iy < ny - 1) put(idx + nx, -fyp);
                if (iz < nz_ - 1) put(idx + nxy, -fzp);
            }
    if (rp) rp[nxy * nz_] = nz;
    return nz;
}

int gen_poisson3d(int nx, int ny, int nz, int* rp, int* ci, double* v) {
    return gen_faces3d(nx, ny, nz, nullptr, rp, ci, v);
}

// k = exp(sigma * g); g: white noise (Box-Muller over SplitMix64) on the grid
// extended by the kernel radius, convolved with the separable kernel
// exp(-d^2/l^2) (whose autocorrelation is the squared-exponential covariance
// exp(-d^2/(2 l^2)) of correlation length l), then shifted and scaled to
// zero mean and unit sample variance.
std::vector<double> gen_log_field(int nx, int ny, int nz, double sigma, double corr, uint64_t seed) {
    const double sk = corr / std::sqrt(2.0);
    const int R = std::max(1, (int)std::ceil(3.0 * sk));
    std::vector<double> ker(2 * R + 1);
    for (int d = -R; d <= R; ++d) ker[d + R] = std::exp(-(double)d * d / (corr * corr));
    const int ex = nx + 2 * R, ey = ny + 2 * R, ez = nz + 2 * R;
    std::vector<double> w((size_t)ex * ey * ez);
    uint64_t rng = seed;
    for (size_t i = 0; i < w.size(); i += 2) {
        const double u1 = 1.0 - u01(rng), u2 = u01(rng);
        const double r = std::sqrt(-2.0 * std::log(u1));
        w[i] = r * std::cos(2.0 * M_PI * u2);
        if (i + 1 < w.size()) w[i + 1] = r * std::sin(2.0 * M_PI * u2);
    }
    // x pass: ex*ey*ez -> nx*ey*ez
    std::vector<double> t1((size_t)nx * ey * ez);
    for (int z = 0; z < ez; ++z)
        for (int y = 0; y < ey; ++y)
            for (int x = 0; x < nx; ++x) {
                double a = 0.0;
                const double* src = &w[((size_t)z * ey + y) * ex + x];
                for (int d = 0; d <= 2 * R; ++d) a += ker[d] * src[d];
                t1[((size_t)z * ey + y) * nx + x] = a;
            }
    std::vector<double>().swap(w);
    std::vector<double> t2((size_t)nx * ny * ez);
    for (int z = 0; z < ez; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                double a = 0.0;
                for (int d = 0; d <= 2 * R; ++d) a += ker[d] * t1[((size_t)z * ey + y + d) * nx + x];
                t2[((size_t)z * ny + y) * nx + x] = a;
            }
    std::vector<double>().swap(t1);
    std::vector<double> g((size_t)nx * ny * nz);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                double a = 0.0;
                for (int d = 0; d <= 2 * R; ++d) a += ker[d] * t2[((size_t)(z + d) * ny + y) * nx + x];
                g[((size_t)z * ny + y) * nx + x] = a;
            }
    double mean = 0.0;
    for (double q : g) mean += q;
    mean /= (double)g.size();
    double var = 0.0;
    for (double q : g) var += (q - mean) * (q - mean);
    var /= (double)g.size();
    const double inv = var > 0 ? 1.0 / std::sqrt(var) : 1.0;
    for (double& q : g) q = std::exp(sigma * (q - mean) * inv);
    return g;
}

int gen_varcoef3d(int nx, int ny, int nz, double sigma, double corr, uint64_t seed, int* rp,
                  int* ci, double* v) {
    if (!rp) return gen_faces3d(nx, ny, nz, nullptr, nullptr, nullptr, nullptr);
    std::vector<double> k = gen_log_field(nx, ny, nz, sigma, corr, seed);
    return gen_faces3d(nx, ny, nz, k.data(), rp, ci, v);
}

void gen_uniform(uint64_t seed, int n, double lo, double hi, double* out) {
    uint64_t rng = seed;
    for (int i = 0; i < n; ++i) out[i] = lo + (hi - lo) * u01(rng);
}

}  // namespace sg
