/* Test infrastructure: the BSIM4v7 half of driver.c's linearisation-point
 * snapshot.  Kept apart because bsim4v7def.h and bsim4def.h both define
 * struct bsim4SizeDependParam.  Not part of the product. */
#include "ngspice/ngspice.h"
#include "ngspice/cktdefs.h"
#include "ngspice/inpdefs.h"
#include "bsim4v7/bsim4v7def.h"
#include "oracle_ref.h"

int oracle_v47_von(void *vckt, double **buf, int *cap, int nv)
{
    CKTcircuit *ckt = (CKTcircuit *)vckt;
    int type = INPtypelook("BSIM4v7");
    BSIM4v7model *model;
    BSIM4v7instance *here;
    if (type < 0)
        return nv;
    for (model = (BSIM4v7model *)ckt->CKThead[type]; model; model = BSIM4v7nextModel(model))
        for (here = BSIM4v7instances(model); here; here = BSIM4v7nextInstance(here)) {
            if (nv >= *cap) {
                *cap = 2 * *cap + 64;
                *buf = TREALLOC(double, *buf, *cap);
            }
            (*buf)[nv++] = here->BSIM4v7von;
        }
    return nv;
}
