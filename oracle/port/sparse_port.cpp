/*
 * Test infrastructure: sparse pivot planning for the CPU oracle port on
 * circuits too large for its dense LU (the C1-size random-logic decks
 * timed as the CPU baseline).  The pivot sequence and the L+U pattern come
 * from the product's host planner (threshold Markowitz, the SMPreorder
 * role of src/maths/KLU/klusmp.c:753-806); the port then re-factors and
 * solves on that pattern in its own C code (port.c).  Nothing in the
 * product links this file.
 */
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../ngspice-sf-mirror_gb300/csrc/circuit.h"
#include "../../ngspice-sf-mirror_gb300/csrc/sparse.h"

extern "C" {

typedef struct {
    int n, nnz, nlu, nlevels, nflevels, nblevels;
    int *a_lupos, *cdiag, *cend, *kptr, *kpos, *kseg, *upd_dst, *upd_src, *prow, *pcol;
    int *lvl_ptr, *lvl_col, *fl_ptr, *fl_row, *bl_ptr, *bl_row;
    int *lr_ptr, *lr_col, *lr_pos, *ur_ptr, *ur_col, *ur_pos;
    int nrl_levels, btf_blocks;   /* right-looking levels; KLU-order blocks */
    double flops;                 /* multiply-adds of one refactorization */
} port_plan_t;

static int *dup(const std::vector<int> &v)
{
    int *p = (int *)malloc(sizeof(int) * (v.size() ? v.size() : 1));
    if (!v.empty())
        memcpy(p, v.data(), sizeof(int) * v.size());
    return p;
}

void port_plan_free(port_plan_t *p)
{
    int **f[] = {&p->a_lupos, &p->cdiag, &p->cend, &p->kptr, &p->kpos, &p->kseg, &p->upd_dst,
                 &p->upd_src, &p->prow, &p->pcol, &p->lvl_ptr, &p->lvl_col, &p->fl_ptr,
                 &p->fl_row, &p->bl_ptr, &p->bl_row, &p->lr_ptr, &p->lr_col, &p->lr_pos,
                 &p->ur_ptr, &p->ur_col, &p->ur_pos};
    for (auto q : f) {
        free(*q);
        *q = nullptr;
    }
}

/* Plan pivots for the n x n CSC matrix (0-based rows).  Returns 0 or -1
 * when the matrix is singular. */
int port_plan(int n, const int *cp, const int *ri, const double *ax, double pivrel,
              double pivtol, port_plan_t *out)
{
    int nnz = cp[n];
    std::vector<int> vcp(cp, cp + n + 1), vri(ri, ri + nnz);
    std::vector<double> vax(ax, ax + nnz);
    ngsf::Image img;
    img.n = n;
    img.a_cp = vcp;
    img.a_ri = vri;
    std::string err;
    if (!ngsf::plan_lu(n, vcp, vri, vax, pivrel, pivtol, img, err))
        return -1;
    port_plan_free(out);
    out->n = n;
    out->nnz = nnz;
    out->nlu = img.nlu;
    out->nlevels = (int)img.lvl_ptr.size() - 1;
    out->nflevels = (int)img.fl_ptr.size() - 1;
    out->nblevels = (int)img.bl_ptr.size() - 1;
    out->nrl_levels = img.rl_ptr.empty() ? 0 : (int)img.rl_ptr.size() - 1;
    out->btf_blocks = img.btf_blocks;
    out->flops = img.lu_flops;
    out->a_lupos = dup(img.a_lupos);
    out->cdiag = dup(img.cdiag);
    out->cend = dup(img.cend);
    out->kptr = dup(img.kptr);
    out->kpos = dup(img.kpos);
    out->kseg = dup(img.kseg);
    out->upd_dst = dup(img.upd_dst);
    out->upd_src = dup(img.upd_src);
    out->prow = dup(img.prow);
    out->pcol = dup(img.pcol);
    out->lvl_ptr = dup(img.lvl_ptr);
    out->lvl_col = dup(img.lvl_col);
    out->fl_ptr = dup(img.fl_ptr);
    out->fl_row = dup(img.fl_row);
    out->bl_ptr = dup(img.bl_ptr);
    out->bl_row = dup(img.bl_row);
    out->lr_ptr = dup(img.lr_ptr);
    out->lr_col = dup(img.lr_col);
    out->lr_pos = dup(img.lr_pos);
    out->ur_ptr = dup(img.ur_ptr);
    out->ur_col = dup(img.ur_col);
    out->ur_pos = dup(img.ur_pos);
    return 0;
}

}  // extern "C"
