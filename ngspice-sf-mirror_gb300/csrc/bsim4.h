/*
 * BSIM4 device image shared by the host compiler (bsim4_setup.cpp) and the
 * GPU load (bsim4_load.cuh).
 *
 * Every quantity the load reads is resolved per instance on the host, in
 * the order BSIM4setup/BSIM4temp produce it (b4set.c, b4temp.c), and stored
 * structure-of-arrays: field f of instance i lives at p[f * n + i].
 */
#ifndef NGSF_BSIM4_H
#define NGSF_BSIM4_H

/* terminals after setup: external d g s b; the internal drain/source
 * primes equal the externals unless series resistance creates them
 * (b4set.c:2437-2530). */
enum { B4N_D, B4N_G, B4N_S, B4N_B, B4N_DP, B4N_SP, B4N_COUNT };

/* per-instance parameters read by the load */
#define B4P_LIST(X)                                                              \
    X(type) X(off) X(icVDS) X(icVGS) X(icVBS) X(vth0) X(vcrit) X(vtm) X(vtm0)     \
    X(SourceSatCurrent) X(DrainSatCurrent) X(Nvtms) X(Nvtmd)                     \
    X(vjsmFwd) X(IVjsmFwd) X(vjdmFwd) X(IVjdmFwd)                                \
    X(Nvtmrss) X(Nvtmrssws) X(Nvtmrsswgs) X(Nvtmrsd) X(Nvtmrsswd) X(Nvtmrsswgd)  \
    X(vtss) X(vtssws) X(vtsswgs) X(vtsd) X(vtsswd) X(vtsswgd)                    \
    X(SjctTempRevSatCur) X(SswTempRevSatCur) X(SswgTempRevSatCur)                \
    X(DjctTempRevSatCur) X(DswTempRevSatCur) X(DswgTempRevSatCur)                \
    X(vbsc) X(phi) X(Xdep0) X(sqrtPhi) X(factor1) X(vbi) X(dvt2) X(dvt2w)        \
    X(dvt1) X(leff) X(dvt0) X(dvt1w) X(weff) X(dvt0w) X(tempRatio) X(lpe0)       \
    X(k1ox) X(kt1) X(kt1l) X(kt2) X(toxe) X(w0) X(eta0) X(etab) X(theta0vb0)     \
    X(lpeb) X(k1) X(k2ox) X(k3) X(k3b) X(coxe) X(cit) X(nfactor) X(cdsc)         \
    X(cdscb) X(cdscd) X(dvtp0) X(dvtp1) X(dvtp4) X(dvtp2factor) X(vfb) X(ngate)  \
    X(mstar) X(voffcbn) X(cdep0) X(dwg) X(dwb) X(prwg) X(prwb) X(rds0)           \
    X(rdswmin) X(nf) X(xj) X(a0) X(b0) X(b1) X(ags) X(keta) X(ketac) X(ua)       \
    X(uc) X(ub) X(ud) X(u0temp) X(vsattemp) X(a1) X(a2) X(delta) X(vtfbphi2)     \
    X(toxp) X(coxp) X(bdos) X(ados) X(fprout) X(pvag) X(pclm) X(litl)            \
    X(thetaRout) X(pdiblb) X(pditsd) X(pdits) X(pditsl) X(pscbe1) X(pscbe2)      \
    X(alpha0) X(alpha1) X(beta0) X(egidl) X(agidl) X(bgidl) X(cgidl) X(weffCJ)   \
    X(egisl) X(agisl) X(bgisl) X(cgisl) X(abulkCVfactor) X(weffCV) X(leffCV)     \
    X(noff) X(voffcv) X(vfbzb) X(acde) X(ldeb) X(moin) X(xpart) X(cgdo) X(cgso)  \
    X(cgbo) X(cgdl) X(cgsl) X(ckappad) X(ckappas)                                \
    X(czbd) X(czbs) X(czbdsw) X(czbdswg) X(czbssw) X(czbsswg)                    \
    X(MJS) X(MJSWS) X(MJSWGS) X(MJD) X(MJSWD) X(MJSWGD)                          \
    X(PhiBS) X(PhiBSWS) X(PhiBSWGS) X(PhiBD) X(PhiBSWD) X(PhiBSWGD)              \
    X(drainConductance) X(sourceConductance) X(m) X(mult_i) X(mult_q)           \
    X(version47)

#define B4P_ENUM(f) B4P_##f,
enum { B4P_LIST(B4P_ENUM) B4P_COUNT };
#undef B4P_ENUM

/* values kept between Newton iterations (here->BSIM4von) */
enum { B4H_VON, B4H_COUNT };

/* state vector layout (bsim4def.h:534-567, 29 doubles) */
enum {
    B4S_VBD, B4S_VBS, B4S_VGS, B4S_VDS, B4S_VDBS, B4S_VDBD, B4S_VSBS, B4S_VGES,
    B4S_VGMS, B4S_VSES, B4S_VDES, B4S_QB, B4S_CQB, B4S_QG, B4S_CQG, B4S_QD,
    B4S_CQD, B4S_QGMID, B4S_CQGMID, B4S_QBS, B4S_CQBS, B4S_QBD, B4S_CQBD,
    B4S_QCHEQ, B4S_CQCHEQ, B4S_QCDUMP, B4S_CQCDUMP, B4S_QDEF, B4S_QS, B4S_COUNT
};

/* Stamps in the order BSIM4LoadRhsMat adds them (b4ld.c:5448-5620) for
 * rgateMod 0, rdsMod 0, rbodyMod 0, trnqsMod 0: four right-hand-side
 * terms, then 38 matrix terms.  Each entry names (row, column) as terminal
 * indices (B4N_*); the slot value already carries the sign of the
 * reference's += / -=. */
#define B4_NSTAMP_RHS 4
#define B4_NSTAMP_MAT 38
#define B4_NSTAMP (B4_NSTAMP_RHS + B4_NSTAMP_MAT)

#endif
