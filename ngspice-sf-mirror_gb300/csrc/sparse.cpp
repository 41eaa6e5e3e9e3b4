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
#include <array>
#include <map>
#include <set>

#include "circuit.h"
#include "sparse.h"

namespace ngsf {

bool plan_lu(int n, const std::vector<int> &cp, const std::vector<int> &ri,
             const std::vector<double> &ax, double pivrel, double pivtol,
             Image &img, std::string &err)
{
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
                for (auto &e : urow[k]) {
                    const int j = e.first, upos = e.second;
                    int q = img.cbeg[j];
                    const int qe = img.cend[j];
                    for (size_t s2 = 0; s2 < lk.size(); s2++) {
                        const int i = lk[s2];
                        while (q < qe && colrow[q] < i)
                            q++;
                        if (q == qe || colrow[q] != i) {
                            err = "internal: fill closure violated (right-looking)";
                            return false;
                        }
                        const int d = q;
                        if (cnt[d]++ == 0)
                            touched.push_back(d);
                        prod.push_back({d, img.cdiag[k] + 1 + (int)s2, upos, img.cdiag[k]});
                    }
                }
            }
            if (touched.size() * 16 > (size_t)img.nlu) {
                /* a dense level: scanning the counts is cheaper than a sort */
                touched.clear();
                for (int d = 0; d < img.nlu; d++)
                    if (cnt[d])
                        touched.push_back(d);
            } else {
                std::sort(touched.begin(), touched.end());
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
