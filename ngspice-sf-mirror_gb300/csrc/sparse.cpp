/*
 * Host symbolic + pivoting analysis of the circuit matrix (the SMPreorder /
 * SMPpreOrder half of the SMP interface, src/maths/KLU/klusmp.c:753-806,
 * 1256-1285).
 *
 * The reference factors with pivoting when NIiter asks for a reorder
 * (MODEINITJCT, first MODEINITTRAN iteration; src/maths/ni/niiter.c:107-146)
 * and re-factors on the fixed pivot sequence otherwise (klu_refactor).  Here
 * the pivoting factorization runs once on the host on the first stamped
 * matrix: a right-looking Markowitz elimination with threshold partial
 * pivoting (a pivot must satisfy |a| >= pivrel * max|column| and
 * |a| > pivtol, the PivRel / PivTol meaning of SMPreorder).  It yields the
 * pivot sequence and the exact fill pattern of L and U.  The GPU then
 * re-factors every Newton iteration on that fixed pattern (engine.cu),
 * left-looking, one column per warp, columns grouped by dependency level.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <array>
#include <map>
#include <set>

#include "circuit.h"
#include "sparse.h"

namespace ngsf {

namespace {

/* Maximum transversal (the zero-free diagonal btf_maxtrans looks for,
 * BTF/Source/btf_maxtrans.c): colRow[j] = the row matched to column j.
 * Cheap passes take each column's own diagonal entry where the pattern has
 * one, then the first free row; every column left unmatched searches
 * depth first for an augmenting path (Duff's MC21).  Keeping the natural
 * diagonal makes the matched entries the MNA diagonal wherever it exists,
 * so the symmetric ordering of each block sees the circuit's own graph
 * (the blocks themselves do not depend on which maximum matching is
 * taken).  Returns false when the matrix is structurally singular. */
bool max_transversal(int n, const std::vector<int> &cp, const std::vector<int> &ri,
                     std::vector<int> &colRow)
{
    std::vector<int> rowCol(n, -1);
    colRow.assign(n, -1);
    for (int j = 0; j < n; j++)
        for (int p = cp[j]; p < cp[j + 1]; p++)
            if (ri[p] == j) {
                rowCol[j] = j;
                colRow[j] = j;
                break;
            }
    for (int j = 0; j < n; j++)
        if (colRow[j] < 0)
            for (int p = cp[j]; p < cp[j + 1]; p++)
                if (rowCol[ri[p]] < 0) {
                    rowCol[ri[p]] = j;
                    colRow[j] = ri[p];
                    break;
                }
    std::vector<int> visited(n, -1);
    std::vector<int> stCol, stPtr, viaRow;   /* viaRow[t]: row leading to stCol[t + 1] */
    for (int j0 = 0; j0 < n; j0++) {
        if (colRow[j0] >= 0)
            continue;
        stCol.assign(1, j0);
        stPtr.assign(1, cp[j0]);
        viaRow.clear();
        visited[j0] = j0;
        int found = -1;
        while (!stCol.empty() && found < 0) {
            const int t = (int)stCol.size() - 1, j = stCol[t];
            bool pushed = false;
            while (stPtr[t] < cp[j + 1]) {
                const int i = ri[stPtr[t]++];
                if (rowCol[i] < 0) {
                    found = i;
                    break;
                }
                const int j2 = rowCol[i];
                if (visited[j2] != j0) {
                    visited[j2] = j0;
                    stCol.push_back(j2);
                    stPtr.push_back(cp[j2]);
                    viaRow.push_back(i);
                    pushed = true;
                    break;
                }
            }
            if (found < 0 && !pushed) {
                stCol.pop_back();
                stPtr.pop_back();
                if (!viaRow.empty())
                    viaRow.pop_back();
            }
        }
        if (found < 0)
            return false;
        /* the last column takes the free row, each earlier one the row
         * through which the path left it */
        for (int t = (int)stCol.size() - 1; t >= 0; t--) {
            const int i = t == (int)stCol.size() - 1 ? found : viaRow[t];
            colRow[stCol[t]] = i;
            rowCol[i] = stCol[t];
        }
    }
    return true;
}

/* Column order of KLU's analysis (klu_analyze.c:451 with btf = TRUE,
 * ordering = AMD): the block upper triangular form from the maximum
 * transversal and the strongly connected components of the matched graph
 * (btf_strongcomp, Tarjan), blocks in topological order; within a block a
 * minimum degree order of the block's symmetrised pattern (AMD's
 * criterion, with exact degrees on the elimination graph; ties by column
 * index).  Q: columns in elimination order; colRow: each column's matched
 * ("diagonal") row; nblocks: the number of diagonal blocks. */
bool btf_md_order(int n, const std::vector<int> &cp, const std::vector<int> &ri,
                  std::vector<int> &Q, std::vector<int> &colRow, int &nblocks,
                  int *largest = nullptr)
{
    if (!max_transversal(n, cp, ri, colRow))
        return false;
    /* rows as lists of columns */
    std::vector<int> rp(n + 1, 0), rc(cp[n]);
    for (int p = 0; p < cp[n]; p++)
        rp[ri[p] + 1]++;
    for (int i = 0; i < n; i++)
        rp[i + 1] += rp[i];
    {
        std::vector<int> fill(rp.begin(), rp.end() - 1);
        for (int j = 0; j < n; j++)
            for (int p = cp[j]; p < cp[j + 1]; p++)
                rc[fill[ri[p]]++] = j;
    }
    /* node j = column j with its matched row; edge j -> k for every entry
     * (colRow[j], k), k != j.  Iterative Tarjan. */
    std::vector<int> index(n, -1), low(n, 0), comp(n, -1), stack;
    std::vector<char> onStack(n, 0);
    std::vector<std::vector<int>> comps;
    int counter = 0;
    std::vector<std::pair<int, int>> call;   /* (node, next entry of its row) */
    for (int s0 = 0; s0 < n; s0++) {
        if (index[s0] >= 0)
            continue;
        call.push_back({s0, rp[colRow[s0]]});
        index[s0] = low[s0] = counter++;
        stack.push_back(s0);
        onStack[s0] = 1;
        while (!call.empty()) {
            const int v = call.back().first;
            const int row = colRow[v];
            bool descended = false;
            while (call.back().second < rp[row + 1]) {
                const int w = rc[call.back().second++];
                if (w == v)
                    continue;
                if (index[w] < 0) {
                    index[w] = low[w] = counter++;
                    stack.push_back(w);
                    onStack[w] = 1;
                    call.push_back({w, rp[colRow[w]]});
                    descended = true;
                    break;
                }
                if (onStack[w])
                    low[v] = std::min(low[v], index[w]);
            }
            if (descended)
                continue;
            if (low[v] == index[v]) {
                std::vector<int> c;
                int w;
                do {
                    w = stack.back();
                    stack.pop_back();
                    onStack[w] = 0;
                    comp[w] = (int)comps.size();
                    c.push_back(w);
                } while (w != v);
                comps.push_back(std::move(c));
            }
            call.pop_back();
            if (!call.empty())
                low[call.back().first] = std::min(low[call.back().first], low[v]);
        }
    }
    /* Tarjan emits a component after every component it reaches: the
     * reverse emission order puts each row's entries at or right of its
     * block (upper block triangular) */
    nblocks = (int)comps.size();
    if (largest) {
        *largest = 0;
        for (auto &c : comps)
            *largest = std::max(*largest, (int)c.size());
    }
    Q.clear();
    Q.reserve(n);
    std::vector<int> local(n, -1);
    for (int b = nblocks - 1; b >= 0; b--) {
        std::vector<int> &c = comps[b];
        std::sort(c.begin(), c.end());
        const int m = (int)c.size();
        if (m == 1) {
            Q.push_back(c[0]);
            continue;
        }
        for (int t = 0; t < m; t++)
            local[c[t]] = t;
        /* symmetrised pattern of the block */
        std::vector<std::vector<int>> adj(m);
        for (int t = 0; t < m; t++) {
            const int j = c[t];
            const int row = colRow[j];
            for (int p = rp[row]; p < rp[row + 1]; p++) {
                const int k = rc[p];
                if (k != j && local[k] >= 0 && comp[k] == b) {
                    adj[t].push_back(local[k]);
                    adj[local[k]].push_back(t);
                }
            }
        }
        std::vector<std::set<int>> g(m);
        for (int t = 0; t < m; t++)
            g[t].insert(adj[t].begin(), adj[t].end());
        std::set<std::pair<int, int>> pq;   /* (degree, local node) */
        for (int t = 0; t < m; t++)
            pq.insert({(int)g[t].size(), t});
        std::vector<char> gone(m, 0);
        while (!pq.empty()) {
            const int v = pq.begin()->second;
            pq.erase(pq.begin());
            gone[v] = 1;
            Q.push_back(c[v]);
            std::vector<int> nb(g[v].begin(), g[v].end());
            for (int u : nb) {
                pq.erase({(int)g[u].size(), u});
                g[u].erase(v);
            }
            for (size_t a = 0; a < nb.size(); a++)
                for (size_t b2 = a + 1; b2 < nb.size(); b2++) {
                    g[nb[a]].insert(nb[b2]);
                    g[nb[b2]].insert(nb[a]);
                }
            for (int u : nb)
                pq.insert({(int)g[u].size(), u});
            g[v].clear();
        }
        for (int t = 0; t < m; t++)
            local[c[t]] = -1;
    }
    return (int)Q.size() == n;
}

}  // namespace

bool btf_analyze(int n, const std::vector<int> &cp, const std::vector<int> &ri, int &nblocks,
                 int &largest)
{
    std::vector<int> Q, colRow;
    return btf_md_order(n, cp, ri, Q, colRow, nblocks, &largest);
}

bool plan_lu(int n, const std::vector<int> &cp, const std::vector<int> &ri,
             const std::vector<double> &ax, double pivrel, double pivtol,
             Image &img, std::string &err)
{
    /* NGSF_ORDER=klu: KLU's pivot sequence instead of threshold Markowitz:
     * columns in the BTF + minimum degree order of the pattern, in each
     * column the matched ("diagonal") row when its row-scaled magnitude is
     * at least pivrel times the column's largest (klu_kernel.c lpivot with
     * Common->tol = PivRel and scale = 2: rows scaled by their largest
     * entry), else the largest */
    const char *ord = getenv("NGSF_ORDER");
    const bool kluOrder = ord && std::string(ord) == "klu";
    std::vector<int> Q, colRow;
    std::vector<double> rscale;
    if (kluOrder) {
        int nb = 0;
        if (!btf_md_order(n, cp, ri, Q, colRow, nb)) {
            err = "structurally singular matrix (no zero-free diagonal)";
            return false;
        }
        rscale.assign(n, 0.0);
        for (int j = 0; j < n; j++)
            for (int p = cp[j]; p < cp[j + 1]; p++)
                rscale[ri[p]] = std::max(rscale[ri[p]], std::fabs(ax[p]));
        img.btf_blocks = nb;
    }

    /* ---------------- numeric Markowitz elimination ------------------ */
    /* active rows: (column, value) in no particular order; active columns:
     * row sets in ascending order (the candidate search visits rows in
     * that order) */
    std::vector<std::vector<std::pair<int, double>>> rows(n);
    std::vector<std::set<int>> cols(n);
    for (int j = 0; j < n; j++)
        for (int p = cp[j]; p < cp[j + 1]; p++) {
            /* columns arrive in ascending order: a repeated (row, column)
             * can only be the row's last entry */
            auto &r = rows[ri[p]];
            if (!r.empty() && r.back().first == j)
                r.back().second += ax[p];
            else
                r.push_back({j, 0.0 + ax[p]});
            cols[j].insert(ri[p]);
        }
    auto val = [&](int i, int j) -> double {
        for (auto &e : rows[i])
            if (e.first == j)
                return e.second;
        return 0.0;
    };
    std::vector<int> colpos(n, -1);   /* scatter of one row: column -> index */
    std::set<std::pair<int, int>> colq;  /* (count, col) */
    for (int j = 0; j < n; j++)
        colq.insert({(int)cols[j].size(), j});
    std::vector<int> prow(n), pcol(n);
    std::vector<std::vector<int>> Lrows(n), Ucols(n);
    std::vector<char> rowDone(n, 0), colDone(n, 0);

    /* rows holding a single entry: a zero-cost (Markowitz) pivot that the
     * column-count search would reach late when its column is long, as for
     * a supply node whose voltage source row is a singleton.  Taking it
     * first keeps the supply's long row and column out of the fill. */
    std::set<int> singles;
    for (int i = 0; i < n; i++)
        if (rows[i].size() == 1)
            singles.insert(i);

    for (int k = 0; k < n; k++) {
        long bestCost = -1;
        int bp = -1, bq = -1;
        double bmag = 0;
        int examined = 0;
        if (kluOrder) {
            const int q = Q[k];
            double amax = 0;
            int imax = -1;
            for (int i : cols[q]) {
                const double a = rscale[i] > 0 ? std::fabs(val(i, q)) / rscale[i] : 0.0;
                if (a > amax) {
                    amax = a;
                    imax = i;
                }
            }
            const int d = colRow[q];
            if (imax >= 0 && cols[q].count(d) && rscale[d] > 0 &&
                std::fabs(val(d, q)) / rscale[d] >= pivrel * amax)
                imax = d;
            if (imax < 0 || !(std::fabs(val(imax, q)) > pivtol)) {
                err = "singular matrix at elimination step " + std::to_string(k);
                return false;
            }
            bp = imax;
            bq = q;
            singles.clear();
        }
        while (!singles.empty()) {
            int i = *singles.begin();
            singles.erase(singles.begin());
            if (rowDone[i] || rows[i].size() != 1)
                continue;
            int q = rows[i][0].first;
            double a = std::fabs(rows[i][0].second);
            double cmax = 0;
            for (int r : cols[q])
                cmax = std::max(cmax, std::fabs(val(r, q)));
            if (cmax > 0 && a >= pivrel * cmax && a > pivtol) {
                bestCost = 0;
                bp = i;
                bq = q;
                bmag = a;
                break;
            }
        }
        for (auto it = colq.begin(); bp < 0 && it != colq.end(); ++it) {
            int q = it->second;
            int cc = it->first;
            if (bestCost >= 0 && (examined >= 6 || (long)(cc - 1) * 0 >= bestCost))
                break;
            if (cc == 0)
                continue;
            double cmax = 0;
            for (int i : cols[q])
                cmax = std::max(cmax, std::fabs(val(i, q)));
            if (!(cmax > 0))
                continue;
            bool found = false;
            for (int i : cols[q]) {
                double a = std::fabs(val(i, q));
                if (a < pivrel * cmax || a <= pivtol)
                    continue;
                long cost = (long)((int)rows[i].size() - 1) * (long)(cc - 1);
                if (bestCost < 0 || cost < bestCost || (cost == bestCost && a > bmag)) {
                    bestCost = cost;
                    bp = i;
                    bq = q;
                    bmag = a;
                }
                found = true;
            }
            if (found)
                examined++;
            if (bestCost == 0)
                break;
        }
        if (bp < 0) {
            err = "singular matrix at elimination step " + std::to_string(k);
            return false;
        }
        int p = bp, q = bq;
        prow[k] = p;
        pcol[k] = q;
        double d = val(p, q);
        /* U row k: columns of row p except q */
        for (auto &e : rows[p])
            if (e.first != q)
                Ucols[k].push_back(e.first);
        std::sort(Ucols[k].begin(), Ucols[k].end());
        /* L column k: rows of column q except p */
        for (int i : cols[q])
            if (i != p)
                Lrows[k].push_back(i);
        /* Schur update: row i's entries scattered by column, so each
         * entry of the pivot row finds its partner in one lookup */
        for (int i : Lrows[k]) {
            auto &r = rows[i];
            const size_t len0 = r.size();
            for (size_t t = 0; t < len0; t++)
                colpos[r[t].first] = (int)t;
            double l = r[colpos[q]].second / d;
            for (auto &e : rows[p]) {
                int j = e.first;
                if (j == q)
                    continue;
                if (colpos[j] < 0) {
                    r.push_back({j, -l * e.second});
                    colq.erase({(int)cols[j].size(), j});
                    cols[j].insert(i);
                    colq.insert({(int)cols[j].size(), j});
                } else {
                    r[colpos[j]].second -= l * e.second;
                }
            }
            for (size_t t = 0; t < len0; t++)
                colpos[r[t].first] = -1;
        }
        /* remove pivot row and column from the active matrix */
        for (auto &e : rows[p]) {
            int j = e.first;
            colq.erase({(int)cols[j].size(), j});
            cols[j].erase(p);
            if (j != q)
                colq.insert({(int)cols[j].size(), j});
        }
        for (int i : Lrows[k]) {
            auto &r = rows[i];
            for (size_t t = 0; t < r.size(); t++)
                if (r[t].first == q) {
                    r[t] = r.back();
                    r.pop_back();
                    break;
                }
            if (r.size() == 1)
                singles.insert(i);
        }
        colq.erase({(int)cols[q].size(), q});
        cols[q].clear();
        rows[p].clear();
        rowDone[p] = colDone[q] = 1;
    }

    /* ---------------- LU layout in pivot order ----------------------- */
    std::vector<int> rpos(n), cpos(n);
    for (int k = 0; k < n; k++) {
        rpos[prow[k]] = k;
        cpos[pcol[k]] = k;
    }
    /* column k: U rows m<k (sorted), diagonal, L rows i>k (sorted) */
    std::vector<std::vector<int>> ucol(n), lcol(n);
    for (int m = 0; m < n; m++)
        for (int j : Ucols[m])
            ucol[cpos[j]].push_back(m);
    for (int k = 0; k < n; k++) {
        for (int i : Lrows[k])
            lcol[k].push_back(rpos[i]);
        std::sort(lcol[k].begin(), lcol[k].end());
        std::sort(ucol[k].begin(), ucol[k].end());
    }
    img.cbeg.assign(n, 0);
    img.cdiag.assign(n, 0);
    img.cend.assign(n, 0);
    int pos = 0;
    for (int k = 0; k < n; k++) {
        img.cbeg[k] = pos;
        pos += (int)ucol[k].size();
        img.cdiag[k] = pos;
        pos += 1;
        pos += (int)lcol[k].size();
        img.cend[k] = pos;
    }
    img.nlu = pos;
    auto posIn = [&](int k, int row) -> int {
        if (row == k)
            return img.cdiag[k];
        if (row < k) {
            auto it = std::lower_bound(ucol[k].begin(), ucol[k].end(), row);
            if (it == ucol[k].end() || *it != row)
                return -1;
            return img.cbeg[k] + (int)(it - ucol[k].begin());
        }
        auto it = std::lower_bound(lcol[k].begin(), lcol[k].end(), row);
        if (it == lcol[k].end() || *it != row)
            return -1;
        return img.cdiag[k] + 1 + (int)(it - lcol[k].begin());
    };

    /* A entries -> LU positions */
    img.a_lupos.assign(ri.size(), -1);
    for (int j = 0; j < n; j++)
        for (int p = cp[j]; p < cp[j + 1]; p++) {
            int q = posIn(cpos[j], rpos[ri[p]]);
            if (q < 0) {
                err = "internal: matrix entry missing from the LU pattern";
                return false;
            }
            img.a_lupos[p] = q;
        }

    /* left-looking update lists and column levels */
    std::vector<int> level(n, 0);
    img.kptr.assign(n + 1, 0);
    img.kdep.clear();
    img.kpos.clear();
    img.kseg.clear();
    img.upd_dst.clear();
    img.upd_src.clear();
    img.kseg.push_back(0);
    double flops = 0;
    /* where[row]: LU position of (row, k) in the current column k, or -1 */
    std::vector<int> where(n, -1);
    for (int k = 0; k < n; k++) {
        for (size_t t = 0; t < ucol[k].size(); t++)
            where[ucol[k][t]] = img.cbeg[k] + (int)t;
        where[k] = img.cdiag[k];
        for (size_t t = 0; t < lcol[k].size(); t++)
            where[lcol[k][t]] = img.cdiag[k] + 1 + (int)t;
        int lv = 0;
        for (size_t t = 0; t < ucol[k].size(); t++) {
            int m = ucol[k][t];
            lv = std::max(lv, level[m] + 1);
            img.kdep.push_back(m);
            img.kpos.push_back(img.cbeg[k] + (int)t);
            for (size_t s = 0; s < lcol[m].size(); s++) {
                int i = lcol[m][s];
                int dst = where[i];
                if (dst < 0) {
                    err = "internal: fill closure violated";
                    return false;
                }
                img.upd_dst.push_back(dst);
                img.upd_src.push_back(img.cdiag[m] + 1 + (int)s);
            }
            flops += (double)lcol[m].size();
            img.kseg.push_back((int)img.upd_dst.size());
        }
        for (int r : ucol[k])
            where[r] = -1;
        where[k] = -1;
        for (int r : lcol[k])
            where[r] = -1;
        flops += (double)lcol[k].size();
        level[k] = lv;
        img.kptr[k + 1] = (int)img.kdep.size();
    }
    img.lu_flops = flops;
    int nlev = 0;
    for (int k = 0; k < n; k++)
        nlev = std::max(nlev, level[k] + 1);
    img.lvl_ptr.assign(nlev + 1, 0);
    for (int k = 0; k < n; k++)
        img.lvl_ptr[level[k] + 1]++;
    for (int l = 0; l < nlev; l++)
        img.lvl_ptr[l + 1] += img.lvl_ptr[l];
    img.lvl_col.assign(n, 0);
    {
        std::vector<int> fill(img.lvl_ptr.begin(), img.lvl_ptr.end() - 1);
        for (int k = 0; k < n; k++)
            img.lvl_col[fill[level[k]]++] = k;
    }

    /* triangular solves, row oriented in pivot order */
    std::vector<std::vector<std::pair<int, int>>> lrow(n), urow(n);
    for (int m = 0; m < n; m++) {
        for (size_t s = 0; s < lcol[m].size(); s++)
            lrow[lcol[m][s]].push_back({m, img.cdiag[m] + 1 + (int)s});
        for (size_t t = 0; t < ucol[m].size(); t++)
            urow[ucol[m][t]].push_back({m, img.cbeg[m] + (int)t});
    }
    img.lr_ptr.assign(n + 1, 0);
    img.ur_ptr.assign(n + 1, 0);
    img.lr_col.clear();
    img.lr_pos.clear();
    img.ur_col.clear();
    img.ur_pos.clear();
    std::vector<int> fl(n, 0), bl(n, 0);
    for (int k = 0; k < n; k++) {
        std::sort(lrow[k].begin(), lrow[k].end());
        for (auto &e : lrow[k]) {
            img.lr_col.push_back(e.first);
            img.lr_pos.push_back(e.second);
            fl[k] = std::max(fl[k], fl[e.first] + 1);
        }
        img.lr_ptr[k + 1] = (int)img.lr_col.size();
    }
    for (int k = 0; k < n; k++) {
        std::sort(urow[k].begin(), urow[k].end());
        for (auto &e : urow[k]) {
            img.ur_col.push_back(e.first);
            img.ur_pos.push_back(e.second);
        }
        img.ur_ptr[k + 1] = (int)img.ur_col.size();
    }
    for (int k = n - 1; k >= 0; k--)
        for (auto &e : urow[k])
            bl[k] = std::max(bl[k], bl[e.first] + 1);
    auto group = [&](const std::vector<int> &lv, std::vector<int> &ptr, std::vector<int> &idx) {
        int nl = 0;
        for (int k = 0; k < n; k++)
            nl = std::max(nl, lv[k] + 1);
        ptr.assign(nl + 1, 0);
        for (int k = 0; k < n; k++)
            ptr[lv[k] + 1]++;
        for (int l = 0; l < nl; l++)
            ptr[l + 1] += ptr[l];
        idx.assign(n, 0);
        std::vector<int> f(ptr.begin(), ptr.end() - 1);
        for (int k = 0; k < n; k++)
            idx[f[lv[k]]++] = k;
    };
    group(fl, img.fl_ptr, img.fl_row);
    group(bl, img.bl_ptr, img.bl_row);

    /* Long rows of the triangular solves (a supply node's U row) are
     * reduced by a warp: per solve level, the rows with more than 32 terms. */
    auto heavy_rows = [&](const std::vector<int> &ptr, const std::vector<int> &rowsv,
                          const std::vector<int> &rp, std::vector<int> &hptr,
                          std::vector<int> &hrow) {
        int nl = (int)ptr.size() - 1;
        hptr.assign(nl + 1, 0);
        hrow.clear();
        for (int l = 0; l < nl; l++) {
            for (int r = ptr[l]; r < ptr[l + 1]; r++) {
                int k = rowsv[r];
                if (rp[k + 1] - rp[k] > 32)
                    hrow.push_back(k);
            }
            hptr[l + 1] = (int)hrow.size();
        }
    };
    heavy_rows(img.fl_ptr, img.fl_row, img.lr_ptr, img.fh_ptr, img.fh_row);
    heavy_rows(img.bl_ptr, img.bl_row, img.ur_ptr, img.bh_ptr, img.bh_row);

    /* Right-looking schedule for large matrices: pivots grouped in levels
     * (a pivot's level is one more than that of every pivot whose column or
     * row it needs); per level, first the L entries of its pivots are
     * divided by the pivots, then every later entry receives the products
     * L(i,k) * U(k,j) of the level's pivots, grouped by destination so that
     * one thread owns each destination.  The critical path is two barriers
     * per level instead of a column's whole dependency chain. */
    {
        std::vector<int> rl(n, 0);
        std::vector<std::vector<int>> lrows_of(n);   /* m with L(k,m) != 0 */
        for (int m = 0; m < n; m++)
            for (int i : lcol[m])
                lrows_of[i].push_back(m);
        for (int k = 0; k < n; k++) {
            int lv = 0;
            for (int m : ucol[k])
                lv = std::max(lv, rl[m] + 1);
            for (int m : lrows_of[k])
                lv = std::max(lv, rl[m] + 1);
            rl[k] = lv;
        }
        int nl = 0;
        for (int k = 0; k < n; k++)
            nl = std::max(nl, rl[k] + 1);
        std::vector<std::vector<int>> piv(nl);
        for (int k = 0; k < n; k++)
            piv[rl[k]].push_back(k);
        img.rl_ptr.assign(nl + 1, 0);
        img.rl_col.clear();
        img.sc_ptr.assign(nl + 1, 0);
        img.sc_pos.clear();
        img.sc_piv.clear();
        img.ud_ptr.assign(nl + 1, 0);
        img.ud_dst.clear();
        img.ud_cptr.assign(1, 0);
        img.ud_l.clear();
        img.ud_u.clear();
        img.ud_p.clear();
        /* the products are those of the left-looking lists, regrouped */
        img.ud_l.reserve(img.upd_dst.size());
        img.ud_u.reserve(img.upd_dst.size());
        img.ud_p.reserve(img.upd_dst.size());
        /* products of one level grouped by destination in ascending
         * position, each group in generation order (a stable counting
         * sort; cnt and start are indexed by LU position) */
        std::vector<int> cnt(img.nlu, 0), start(img.nlu, 0), touched;
        /* destinations touched in the level, one bit per LU position:
         * enumerating the set bits gives them in ascending order */
        std::vector<uint64_t> mark((size_t)img.nlu / 64 + 1, 0);
        std::vector<int> colrow(img.nlu);   /* row of each LU position */
        for (int j = 0; j < n; j++) {
            for (size_t t = 0; t < ucol[j].size(); t++)
                colrow[img.cbeg[j] + t] = ucol[j][t];
            colrow[img.cdiag[j]] = j;
            for (size_t t = 0; t < lcol[j].size(); t++)
                colrow[img.cdiag[j] + 1 + t] = lcol[j][t];
        }
        std::vector<std::array<int, 4>> prod;   /* dst, lpos, upos, pivot */
        for (int l = 0; l < nl; l++) {
            prod.clear();
            touched.clear();
            for (int k : piv[l]) {
                img.rl_col.push_back(k);
                for (size_t s2 = 0; s2 < lcol[k].size(); s2++) {
                    img.sc_pos.push_back(img.cdiag[k] + 1 + (int)s2);
                    img.sc_piv.push_back(img.cdiag[k]);
                }
                /* per U entry (k, j): the rows of L column k located in
                 * column j by one merge walk (column j's rows are sorted
                 * by position); within a destination the products keep
                 * the pivot order, whatever the walk order */
                const std::vector<int> &lk = lcol[k];
                if (lk.empty())
                    continue;
                for (auto &e : urow[k]) {
                    const int j = e.first, upos = e.second;
                    const int qe = img.cend[j];
                    /* column j's rows ascend with the position: start the
                     * walk at the first row not below L column k's first */
                    int q = (int)(std::lower_bound(colrow.begin() + img.cbeg[j],
                                                   colrow.begin() + qe, lk[0]) -
                                  colrow.begin());
                    for (size_t s2 = 0; s2 < lk.size(); s2++) {
                        const int i = lk[s2];
                        while (q < qe && colrow[q] < i)
                            q++;
                        if (q == qe || colrow[q] != i) {
                            err = "internal: fill closure violated (right-looking)";
                            return false;
                        }
                        const int d = q;
                        if (cnt[d]++ == 0) {
                            touched.push_back(d);
                            mark[(size_t)d >> 6] |= 1ull << (d & 63);
                        }
                        prod.push_back({d, img.cdiag[k] + 1 + (int)s2, upos, img.cdiag[k]});
                    }
                }
            }
            if (!touched.empty()) {
                /* ascending destinations from the bit marks (cleared on the
                 * way), between the smallest and largest touched word */
                size_t w0 = (size_t)-1, w1 = 0;
                for (int d : touched) {
                    w0 = std::min(w0, (size_t)d >> 6);
                    w1 = std::max(w1, (size_t)d >> 6);
                }
                touched.clear();
                for (size_t w = w0; w <= w1; w++) {
                    uint64_t m = mark[w];
                    mark[w] = 0;
                    while (m) {
                        const int b = __builtin_ctzll(m);
                        touched.push_back((int)(w * 64 + (size_t)b));
                        m &= m - 1;
                    }
                }
            }
            const int base = (int)img.ud_l.size();
            int off = base;
            for (int d : touched) {
                start[d] = off;
                off += cnt[d];
                img.ud_dst.push_back(d);
                img.ud_cptr.push_back(off);
                cnt[d] = 0;
            }
            img.ud_l.resize(off);
            img.ud_u.resize(off);
            img.ud_p.resize(off);
            for (auto &c : prod) {
                const int at = start[c[0]]++;
                img.ud_l[at] = c[1];
                img.ud_u[at] = c[2];
                img.ud_p[at] = c[3];
            }
            img.rl_ptr[l + 1] = (int)img.rl_col.size();
            img.sc_ptr[l + 1] = (int)img.sc_pos.size();
            img.ud_ptr[l + 1] = (int)img.ud_dst.size();
        }
    }

    img.prow.resize(n);
    img.pcol.resize(n);
    for (int k = 0; k < n; k++) {
        img.prow[k] = prow[k] + 1;
        img.pcol[k] = pcol[k] + 1;
    }
    return true;
}

}  // namespace ngsf
