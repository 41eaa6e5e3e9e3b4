/*
 * BSIM4 load of one instance (included by bsim4_load.cuh after the engine's
 * Ctl/Iter context and the devsup limiting helpers are defined).
 *
 * Section comments give the b4ld.c lines each block restates.
 */

/* Load one instance.  P points at the instance's first parameter (field f
 * at P[f * ps]), H at its first memory (stride hs), node[] holds its six
 * equation numbers (B4N_*), st its state offset; the 42 stamp values go to
 * sv[k * svs].  Returns 1 when limiting leaves the instance unconverged. */
NGSF_HD inline int bsim4_eval(const B4Ctx &x, const double *P, size_t ps, double *H, size_t hs,
                              const int *node, int st, double *sv, size_t svs)
{
#define Q(f) P[(size_t)B4P_##f * ps]
    const int mode = x.mode;
    const int dN = node[B4N_D], gN = node[B4N_G];
    const int sN = node[B4N_S], bN = node[B4N_B];
    const int dpN = node[B4N_DP], spN = node[B4N_SP];
    double *st0 = x.st0 + st;
    double *st1 = x.st1 + st;
    const double *st2 = x.st2 + st;
    const double type = Q(type);
    const bool off = Q(off) != 0.0;
    const double gmin = x.gmin;
    const bool ccn = (mode & (NGSF_MODEDCTRANCURVE | NGSF_MODETRAN)) != 0;
    int Check = 1;

    /* ---- terminal voltages: initialisation, predictor, limiting
     *      (b4ld.c:256-690) ---- */
    double vds, vgs, vbs, vges, vgms, vdbs, vsbs, vses, vdes;
    if (mode & NGSF_MODEINITTRAN) {
        vds = st1[B4S_VDS];
        vgs = st1[B4S_VGS];
        vbs = st1[B4S_VBS];
        vges = st1[B4S_VGES];
        vgms = st1[B4S_VGMS];
        vdbs = st1[B4S_VDBS];
        vsbs = st1[B4S_VSBS];
        vses = st1[B4S_VSES];
        vdes = st1[B4S_VDES];
    } else if ((mode & NGSF_MODEINITJCT) && !off) {
        vds = type * Q(icVDS);
        vgs = vges = vgms = type * Q(icVGS);
        vbs = vdbs = vsbs = type * Q(icVBS);
        if (vds > 0.0) {
            vdes = vds + 0.01;
            vses = -0.01;
        } else if (vds < 0.0) {
            vdes = vds - 0.01;
            vses = 0.01;
        } else {
            vdes = vses = 0.0;
        }
        if ((vds == 0.0) && (vgs == 0.0) && (vbs == 0.0) &&
            ((mode & (NGSF_MODETRAN | NGSF_MODEDCOP | NGSF_MODEDCTRANCURVE)) ||
             (!(mode & NGSF_MODEUIC)))) {
            vds = 0.1;
            vdes = 0.11;
            vses = -0.01;
            vgs = vges = vgms = type * Q(vth0) + 0.1;
            vbs = vdbs = vsbs = 0.0;
        }
    } else if ((mode & (NGSF_MODEINITJCT | NGSF_MODEINITFIX)) && off) {
        vds = vgs = vbs = vges = vgms = 0.0;
        vdbs = vsbs = vdes = vses = 0.0;
    } else {
        if (mode & NGSF_MODEINITPRED) {
            const double xfact = x.delta / x.deltaOld1;
#define B4PRED(slot, var)                                                   \
    st0[slot] = st1[slot];                                                  \
    var = (1.0 + xfact) * (st1[slot]) - (xfact * (st2[slot]));
            B4PRED(B4S_VDS, vds)
            B4PRED(B4S_VGS, vgs)
            B4PRED(B4S_VGES, vges)
            B4PRED(B4S_VGMS, vgms)
            B4PRED(B4S_VBS, vbs)
            st0[B4S_VBD] = st0[B4S_VBS] - st0[B4S_VDS];
            B4PRED(B4S_VDBS, vdbs)
            st0[B4S_VDBD] = st0[B4S_VDBS] - st0[B4S_VDS];
            B4PRED(B4S_VSBS, vsbs)
            B4PRED(B4S_VSES, vses)
            B4PRED(B4S_VDES, vdes)
            st0[B4S_QDEF] = st1[B4S_QDEF];
#undef B4PRED
        }
        if (!(mode & NGSF_MODEINITPRED) || (mode & NGSF_MODEGUESS)) {
            /* INITFLOAT, or a predictor guess in rhsOld (after the
             * INITPRED state copies above) */
            const double *ro = x.rhsOld;
            vds = type * (ro[dpN] - ro[spN]);
            vgs = type * (ro[gN] - ro[spN]);
            vbs = type * (ro[bN] - ro[spN]);
            vges = type * (ro[gN] - ro[spN]);
            vgms = type * (ro[gN] - ro[spN]);
            vdbs = type * (ro[bN] - ro[spN]);
            vsbs = type * (ro[bN] - ro[spN]);
            vses = type * (ro[sN] - ro[spN]);
            vdes = type * (ro[dN] - ro[spN]);
        }
        const double vgdo = st0[B4S_VGS] - st0[B4S_VDS];
        double vbd = vbs - vds;     /* before limiting, as b4ld.c:444 */
        double vgd = vgs - vds;
        const double von = H[(size_t)B4H_VON * hs];
        if (st0[B4S_VDS] >= 0.0) {
            vgs = dev_fetlim(vgs, st0[B4S_VGS], von);
            vds = vgs - vgd;
            vds = dev_limvds(vds, st0[B4S_VDS]);
            vgd = vgs - vds;
        } else {
            vgd = dev_fetlim(vgd, vgdo, von);
            vds = vgs - vgd;
            vds = -dev_limvds(-vds, -(st0[B4S_VDS]));
            vgs = vgd + vds;
        }
        if (vds >= 0.0) {
            vbs = dev_pnjlim(vbs, st0[B4S_VBS], B4_CONSTVT0, Q(vcrit), &Check);
        } else {
            vbd = dev_pnjlim(vbd, st0[B4S_VBD], B4_CONSTVT0, Q(vcrit), &Check);
            vbs = vbd + vds;
        }
    }
    const double qdef = 0.0;    /* type * rhsOld[qNode = ground] */

    /* ---- DC currents (b4ld.c:692-1003) ---- */
    const double vbd = vbs - vds;
    const double vgd = vgs - vds;
    const double vgb = vgs - vbs;
    const double vdbd = vdbs - vds;
    const double vbs_jct = vbs;
    const double vbd_jct = vbd;
    (void)vges; (void)vgms;

    double gbs, cbs, gbd, cbd;
    b4_junction_dio1(Q(SourceSatCurrent), Q(Nvtms), Q(vjsmFwd), Q(IVjsmFwd), vbs_jct, gmin,
                     gbs, cbs);
    b4_junction_dio1(Q(DrainSatCurrent), Q(Nvtmd), Q(vjdmFwd), Q(IVjdmFwd), vbd_jct, gmin,
                     gbd, cbd);
    {
        double T1, T2, T3, T4, T5, T6, d1, d2, d3, d4, d5, d6;
        b4_tat(Q(vtss), Q(Nvtmrss), vbs_jct, T1, d1);
        b4_tat(Q(vtsd), Q(Nvtmrsd), vbd_jct, T2, d2);
        b4_tat(Q(vtssws), Q(Nvtmrssws), vbs_jct, T3, d3);
        b4_tat(Q(vtsswd), Q(Nvtmrsswd), vbd_jct, T4, d4);
        b4_tat(Q(vtsswgs), Q(Nvtmrsswgs), vbs_jct, T5, d5);
        b4_tat(Q(vtsswgd), Q(Nvtmrsswgd), vbd_jct, T6, d6);
        gbs += Q(SjctTempRevSatCur) * d1 + Q(SswTempRevSatCur) * d3 + Q(SswgTempRevSatCur) * d5;
        cbs -= Q(SjctTempRevSatCur) * (T1 - 1.0) + Q(SswTempRevSatCur) * (T3 - 1.0) +
               Q(SswgTempRevSatCur) * (T5 - 1.0);
        gbd += Q(DjctTempRevSatCur) * d2 + Q(DswTempRevSatCur) * d4 + Q(DswgTempRevSatCur) * d6;
        cbd -= Q(DjctTempRevSatCur) * (T2 - 1.0) + Q(DswTempRevSatCur) * (T4 - 1.0) +
               Q(DswgTempRevSatCur) * (T6 - 1.0);
    }

    int bmode;
    double Vds, Vgs, Vbs;
    if (vds >= 0.0) {
        bmode = 1;
        Vds = vds;
        Vgs = vgs;
        Vbs = vbs;
    } else {
        bmode = -1;
        Vds = -vds;
        Vgs = vgd;
        Vbs = vbd;
    }
    (void)Vgs;
    const double toxe = Q(toxe);
    const double epssub = B4_EPSSI;

    /* Vbseff (b4ld.c:1033-1052) */
    double T0, T1, T2, T3, T4, T5, T6, T7, T8, T9, T10, T11, T12, T13;
    double tmp1, tmp2, tmp3, tmp4;
    const double vbsc = Q(vbsc);
    double Vbseff, dVbseff_dVb;
    T0 = Vbs - vbsc - 0.001;
    T1 = sqrt(T0 * T0 - 0.004 * vbsc);
    if (T0 >= 0.0) {
        Vbseff = vbsc + 0.5 * (T0 + T1);
        dVbseff_dVb = 0.5 * (1.0 + T0 / T1);
    } else {
        T2 = -0.002 / (T1 - T0);
        Vbseff = vbsc * (1.0 + T2);
        dVbseff_dVb = T2 * vbsc / T1;
    }
    const double phi = Q(phi), sqrtPhi = Q(sqrtPhi);
    T9 = 0.95 * phi;
    T0 = T9 - Vbseff - 0.001;
    T1 = sqrt(T0 * T0 + 0.004 * T9);
    Vbseff = T9 - 0.5 * (T0 + T1);
    dVbseff_dVb *= 0.5 * (1.0 + T0 / T1);
    const double Phis = phi - Vbseff;
    const double dPhis_dVb = -1.0;
    const double sqrtPhis = sqrt(Phis);
    const double dsqrtPhis_dVb = -0.5 / sqrtPhis;
    const double Xdep0 = Q(Xdep0);
    const double Xdep = Xdep0 * sqrtPhis / sqrtPhi;
    const double dXdep_dVb = (Xdep0 / sqrtPhi) * dsqrtPhis_dVb;
    const double Leff = Q(leff);
    const double Vtm = Q(vtm);

    /* threshold voltage (b4ld.c:1063-1200) */
    T3 = sqrt(Xdep);
    const double V0 = Q(vbi) - phi;
    const double factor1 = Q(factor1);
    const double dvt2 = Q(dvt2), dvt2w = Q(dvt2w);
    T0 = dvt2 * Vbseff;
    if (T0 >= -0.5) {
        T1 = 1.0 + T0;
        T2 = dvt2;
    } else {
        T4 = 1.0 / (3.0 + 8.0 * T0);
        T1 = (1.0 + 3.0 * T0) * T4;
        T2 = dvt2 * T4 * T4;
    }
    const double lt1 = factor1 * T3 * T1;
    const double dlt1_dVb = factor1 * (0.5 / T3 * T1 * dXdep_dVb + T3 * T2);
    T0 = dvt2w * Vbseff;
    if (T0 >= -0.5) {
        T1 = 1.0 + T0;
        T2 = dvt2w;
    } else {
        T4 = 1.0 / (3.0 + 8.0 * T0);
        T1 = (1.0 + 3.0 * T0) * T4;
        T2 = dvt2w * T4 * T4;
    }
    const double ltw = factor1 * T3 * T1;
    const double dltw_dVb = factor1 * (0.5 / T3 * T1 * dXdep_dVb + T3 * T2);
    double Theta0, dTheta0_dVb, dT1_dVb;
    T0 = Q(dvt1) * Leff / lt1;
    if (T0 < B4_EXP_THRESHOLD) {
        T1 = exp(T0);
        T2 = T1 - 1.0;
        T3 = T2 * T2;
        T4 = T3 + 2.0 * T1 * B4_MIN_EXP;
        Theta0 = T1 / T4;
        dT1_dVb = -T0 * T1 * dlt1_dVb / lt1;
        dTheta0_dVb = dT1_dVb * (T4 - 2.0 * T1 * (T2 + B4_MIN_EXP)) / T4 / T4;
    } else {
        Theta0 = 1.0 / (B4_MAX_EXP - 2.0);
        dTheta0_dVb = 0.0;
    }
    const double thetavth = Q(dvt0) * Theta0;
    const double Delt_vth = thetavth * V0;
    const double dDelt_vth_dVb = Q(dvt0) * dTheta0_dVb * V0;
    double dT5_dVb;
    T0 = Q(dvt1w) * Q(weff) * Leff / ltw;
    if (T0 < B4_EXP_THRESHOLD) {
        T1 = exp(T0);
        T2 = T1 - 1.0;
        T3 = T2 * T2;
        T4 = T3 + 2.0 * T1 * B4_MIN_EXP;
        T5 = T1 / T4;
        dT1_dVb = -T0 * T1 * dltw_dVb / ltw;
        dT5_dVb = dT1_dVb * (T4 - 2.0 * T1 * (T2 + B4_MIN_EXP)) / T4 / T4;
    } else {
        T5 = 1.0 / (B4_MAX_EXP - 2.0);
        dT5_dVb = 0.0;
    }
    T0 = Q(dvt0w) * T5;
    T2 = T0 * V0;
    const double dT2_dVb_w = Q(dvt0w) * dT5_dVb * V0;
    const double TempRatio = Q(tempRatio);
    T0 = sqrt(1.0 + Q(lpe0) / Leff);
    const double k1ox = Q(k1ox), k1 = Q(k1), k3b = Q(k3b);
    T1 = k1ox * (T0 - 1.0) * sqrtPhi + (Q(kt1) + Q(kt1l) / Leff + Q(kt2) * Vbseff) * TempRatio;
    const double Vth_NarrowW = toxe * phi / (Q(weff) + Q(w0));
    T3 = Q(eta0) + Q(etab) * Vbseff;
    if (T3 < 1.0e-4) {
        T9 = 1.0 / (3.0 - 2.0e4 * T3);
        T3 = (2.0e-4 - T3) * T9;
        T4 = T9 * T9;
    } else {
        T4 = 1.0;
    }
    const double theta0vb0 = Q(theta0vb0);
    const double dDIBL_Sft_dVd = T3 * theta0vb0;
    const double DIBL_Sft = dDIBL_Sft_dVd * Vds;
    const double Lpe_Vb = sqrt(1.0 + Q(lpeb) / Leff);
    const double k2ox = Q(k2ox);
    double Vth = type * Q(vth0) + (k1ox * sqrtPhis - k1 * sqrtPhi) * Lpe_Vb - k2ox * Vbseff -
                 Delt_vth - T2 + (Q(k3) + k3b * Vbseff) * Vth_NarrowW + T1 - DIBL_Sft;
    double dVth_dVb = Lpe_Vb * k1ox * dsqrtPhis_dVb - k2ox - dDelt_vth_dVb - dT2_dVb_w +
                      k3b * Vth_NarrowW - Q(etab) * Vds * theta0vb0 * T4 + Q(kt2) * TempRatio;
    double dVth_dVd = -dDIBL_Sft_dVd;

    /* subthreshold swing n (b4ld.c:1147-1168) */
    const double coxe = Q(coxe);
    tmp1 = epssub / Xdep;
    tmp2 = Q(nfactor) * tmp1;
    tmp3 = Q(cdsc) + Q(cdscb) * Vbseff + Q(cdscd) * Vds;
    tmp4 = (tmp2 + tmp3 * Theta0 + Q(cit)) / coxe;
    double n_, dn_dVb, dn_dVd;
    if (tmp4 >= -0.5) {
        n_ = 1.0 + tmp4;
        dn_dVb = (-tmp2 / Xdep * dXdep_dVb + tmp3 * dTheta0_dVb + Q(cdscb) * Theta0) / coxe;
        dn_dVd = Q(cdscd) * Theta0 / coxe;
    } else {
        T0 = 1.0 / (3.0 + 8.0 * tmp4);
        n_ = (1.0 + 3.0 * tmp4) * T0;
        T0 *= T0;
        dn_dVb = (-tmp2 / Xdep * dXdep_dVb + tmp3 * dTheta0_dVb + Q(cdscb) * Theta0) / coxe * T0;
        dn_dVd = Q(cdscd) * Theta0 / coxe * T0;
    }

    /* pocket-implant and DITS shifts (b4ld.c:1170-1222) */
    if (Q(dvtp0) > 0.0) {
        double dT2_dVd;
        T0 = -Q(dvtp1) * Vds;
        if (T0 < -B4_EXP_THRESHOLD) {
            T2 = B4_MIN_EXP;
            dT2_dVd = 0.0;
        } else {
            T2 = exp(T0);
            dT2_dVd = -Q(dvtp1) * T2;
        }
        T3 = Leff + Q(dvtp0) * (1.0 + T2);
        const double dT3_dVd = Q(dvtp0) * dT2_dVd;
        T4 = Vtm * log(Leff / T3);
        const double dT4_dVd = -Vtm * dT3_dVd / T3;
        const double dDITS_Sft_dVd = dn_dVd * T4 + n_ * dT4_dVd;
        const double dDITS_Sft_dVb = T4 * dn_dVb;
        Vth -= n_ * T4;
        dVth_dVd -= dDITS_Sft_dVd;
        dVth_dVb -= dDITS_Sft_dVb;
    }
    if ((Q(dvtp4) == 0.0) || (Q(dvtp2factor) == 0.0)) {
        /* no DITS_Sft2 */
    } else {
        T1 = 2.0 * Q(dvtp4) * Vds;
        b4_dexp(T1, T0, T10);
        const double DITS_Sft2 = Q(dvtp2factor) * (T0 - 1) / (T0 + 1);
        const double dDITS_Sft2_dVd = Q(dvtp2factor) * Q(dvtp4) * 4.0 * T10 / ((T0 + 1) * (T0 + 1));
        Vth -= DITS_Sft2;
        dVth_dVd -= dDITS_Sft2_dVd;
    }
    H[(size_t)B4H_VON * hs] = Vth;

    /* poly-gate depletion (b4ld.c:1226-1247) */
    double vgs_eff, dvgs_eff_dvg, vgd_eff, dvgd_eff_dvg;
    T0 = Q(vfb) + phi;
    b4_poly_depletion(T0, Q(ngate), B4_EPSSI, coxe, vgs, vgs_eff, dvgs_eff_dvg);
    b4_poly_depletion(T0, Q(ngate), B4_EPSSI, coxe, vgd, vgd_eff, dvgd_eff_dvg);
    double Vgs_eff, dVgs_eff_dVg;
    if (bmode > 0) {
        Vgs_eff = vgs_eff;
        dVgs_eff_dVg = dvgs_eff_dvg;
    } else {
        Vgs_eff = vgd_eff;
        dVgs_eff_dVg = dvgd_eff_dvg;
    }
    const double Vgst = Vgs_eff - Vth;

    /* Vgsteff (b4ld.c:1249-1306) */
    const double mstar = Q(mstar);
    double dT10_dVg, dT10_dVd, dT10_dVb, dT9_dVg, dT9_dVd, dT9_dVb, ExpVgst;
    T0 = n_ * Vtm;
    T1 = mstar * Vgst;
    T2 = T1 / T0;
    if (T2 > B4_EXP_THRESHOLD) {
        T10 = T1;
        dT10_dVg = mstar * dVgs_eff_dVg;
        dT10_dVd = -dVth_dVd * mstar;
        dT10_dVb = -dVth_dVb * mstar;
    } else if (T2 < -B4_EXP_THRESHOLD) {
        T10 = Vtm * log(1.0 + B4_MIN_EXP);
        dT10_dVg = 0.0;
        dT10_dVd = T10 * dn_dVd;
        dT10_dVb = T10 * dn_dVb;
        T10 *= n_;
    } else {
        ExpVgst = exp(T2);
        T3 = Vtm * log(1.0 + ExpVgst);
        T10 = n_ * T3;
        dT10_dVg = mstar * ExpVgst / (1.0 + ExpVgst);
        dT10_dVb = T3 * dn_dVb - dT10_dVg * (dVth_dVb + Vgst * dn_dVb / n_);
        dT10_dVd = T3 * dn_dVd - dT10_dVg * (dVth_dVd + Vgst * dn_dVd / n_);
        dT10_dVg *= dVgs_eff_dVg;
    }
    T1 = Q(voffcbn) - (1.0 - mstar) * Vgst;
    T2 = T1 / T0;
    if (T2 < -B4_EXP_THRESHOLD) {
        T3 = coxe * B4_MIN_EXP / Q(cdep0);
        T9 = mstar + T3 * n_;
        dT9_dVg = 0.0;
        dT9_dVd = dn_dVd * T3;
        dT9_dVb = dn_dVb * T3;
    } else if (T2 > B4_EXP_THRESHOLD) {
        T3 = coxe * B4_MAX_EXP / Q(cdep0);
        T9 = mstar + T3 * n_;
        dT9_dVg = 0.0;
        dT9_dVd = dn_dVd * T3;
        dT9_dVb = dn_dVb * T3;
    } else {
        ExpVgst = exp(T2);
        T3 = coxe / Q(cdep0);
        T4 = T3 * ExpVgst;
        T5 = T1 * T4 / T0;
        T9 = mstar + n_ * T4;
        dT9_dVg = T3 * (mstar - 1.0) * ExpVgst / Vtm;
        dT9_dVb = T4 * dn_dVb - dT9_dVg * dVth_dVb - T5 * dn_dVb;
        dT9_dVd = T4 * dn_dVd - dT9_dVg * dVth_dVd - T5 * dn_dVd;
        dT9_dVg *= dVgs_eff_dVg;
    }
    double Vgsteff = T10 / T9;
    T11 = T9 * T9;
    double dVgsteff_dVg = (T9 * dT10_dVg - T10 * dT9_dVg) / T11;
    double dVgsteff_dVd = (T9 * dT10_dVd - T10 * dT9_dVd) / T11;
    double dVgsteff_dVb = (T9 * dT10_dVb - T10 * dT9_dVb) / T11;

    /* effective width and Rds, rdsMod 0 (b4ld.c:1308-1350) */
    T9 = sqrtPhis - sqrtPhi;
    double Weff = Q(weff) - 2.0 * (Q(dwg) * Vgsteff + Q(dwb) * T9);
    double dWeff_dVg = -2.0 * Q(dwg);
    double dWeff_dVb = -2.0 * Q(dwb) * dsqrtPhis_dVb;
    if (Weff < 2.0e-8) {
        T0 = 1.0 / (6.0e-8 - 2.0 * Weff);
        Weff = 2.0e-8 * (4.0e-8 - Weff) * T0;
        T0 *= T0 * 4.0e-16;
        dWeff_dVg *= T0;
        dWeff_dVb *= T0;
    }
    double Rds, dRds_dVg, dRds_dVb;
    {
        T0 = 1.0 + Q(prwg) * Vgsteff;
        const double dT0_dVg = -Q(prwg) / T0 / T0;
        T1 = Q(prwb) * T9;
        dT1_dVb = Q(prwb) * dsqrtPhis_dVb;
        T2 = 1.0 / T0 + T1;
        T3 = T2 + sqrt(T2 * T2 + 0.01);
        double dT3_dVg = 1.0 + T2 / (T3 - T2);
        const double dT3_dVb = dT3_dVg * dT1_dVb;
        dT3_dVg *= dT0_dVg;
        T4 = Q(rds0) * 0.5;
        Rds = Q(rdswmin) + T3 * T4;
        dRds_dVg = T4 * dT3_dVg;
        dRds_dVb = T4 * dT3_dVb;
    }

    /* bulk charge factor Abulk (b4ld.c:1352-1440) */
    T9 = 0.5 * k1ox * Lpe_Vb / sqrtPhis;
    T1 = T9 + k2ox - k3b * Vth_NarrowW;
    dT1_dVb = -T9 / sqrtPhis * dsqrtPhis_dVb;
    T9 = sqrt(Q(xj) * Xdep);
    tmp1 = Leff + 2.0 * T9;
    T5 = Leff / tmp1;
    tmp2 = Q(a0) * T5;
    tmp3 = Q(weff) + Q(b1);
    tmp4 = Q(b0) / tmp3;
    T2 = tmp2 + tmp4;
    const double dT2_dVb = -T9 / tmp1 / Xdep * dXdep_dVb;
    T6 = T5 * T5;
    T7 = T5 * T6;
    double Abulk0 = 1.0 + T1 * T2;
    double dAbulk0_dVb = T1 * tmp2 * dT2_dVb + T2 * dT1_dVb;
    T8 = Q(ags) * Q(a0) * T7;
    double dAbulk_dVg = -T1 * T8;
    double Abulk = Abulk0 + dAbulk_dVg * Vgsteff;
    double dAbulk_dVb = dAbulk0_dVb - T8 * Vgsteff * (dT1_dVb + 3.0 * T1 * dT2_dVb);
    if (Abulk0 < 0.1) {
        T9 = 1.0 / (3.0 - 20.0 * Abulk0);
        Abulk0 = (0.2 - Abulk0) * T9;
        dAbulk0_dVb *= T9 * T9;
    }
    if (Abulk < 0.1) {
        T9 = 1.0 / (3.0 - 20.0 * Abulk);
        Abulk = (0.2 - Abulk) * T9;
        T10 = T9 * T9;
        dAbulk_dVb *= T10;
        dAbulk_dVg *= T10;
    }
    double dT0_dVb;
    const double keta = Q(keta), ketac = Q(ketac);
    T2 = keta * Vbseff;
    if (T2 >= -0.9) {
        T0 = 1.0 / (1.0 + T2);
        dT0_dVb = -keta * T0 * T0;
    } else {
        T1 = 1.0 / (0.8 + T2);
        T0 = (17.0 + 20.0 * T2) * T1;
        dT0_dVb = -keta * T1 * T1;
    }
    dAbulk_dVg *= T0;
    dAbulk_dVb = dAbulk_dVb * T0 + Abulk * dT0_dVb;
    double dAbulk0_Q_dVb = dAbulk0_dVb;
    dAbulk0_dVb = dAbulk0_dVb * T0 + Abulk0 * dT0_dVb;
    Abulk *= T0;
    double Abulk0_Q = Abulk0;
    Abulk0 *= T0;
    if (ketac != keta) {
        T2 = ketac * Vbseff;
        if (T2 >= -0.9) {
            T0 = 1.0 / (1.0 + T2);
            dT0_dVb = -ketac * T0 * T0;
        } else {
            T1 = 1.0 / (0.8 + T2);
            T0 = (17.0 + 20.0 * T2) * T1;
            dT0_dVb = -ketac * T1 * T1;
        }
        dAbulk0_Q_dVb = dAbulk0_Q_dVb * T0 + Abulk0_Q * dT0_dVb;
        Abulk0_Q *= T0;
    } else {
        dAbulk0_Q_dVb = dAbulk0_dVb;
        Abulk0_Q = Abulk0;
    }

    /* mobility, mobMod 0 (b4ld.c:1448-1470, 1595-1612) */
    double dDenomi_dVg, dDenomi_dVd, dDenomi_dVb, Denomi;
    {
        const double T14 = 0.0;
        T0 = Vgsteff + Vth + Vth - T14;
        T2 = Q(ua) + Q(uc) * Vbseff;
        T3 = T0 / toxe;
        T12 = sqrt(Vth * Vth + 0.0001);
        T9 = 1.0 / (Vgsteff + 2 * T12);
        T10 = T9 * toxe;
        T8 = Q(ud) * T10 * T10 * Vth;
        T6 = T8 * Vth;
        T5 = T3 * (T2 + Q(ub) * T3) + T6;
        T7 = -2.0 * T6 * T9;
        T11 = T7 * Vth / T12;
        dDenomi_dVg = (T2 + 2.0 * Q(ub) * T3) / toxe;
        T13 = 2.0 * (dDenomi_dVg + T11 + T8);
        dDenomi_dVd = T13 * dVth_dVd;
        dDenomi_dVb = T13 * dVth_dVb + Q(uc) * T3;
        dDenomi_dVg += T7;
    }
    if (T5 >= -0.8) {
        Denomi = 1.0 + T5;
    } else {
        T9 = 1.0 / (7.0 + 10.0 * T5);
        Denomi = (0.6 + T5) * T9;
        T9 *= T9;
        dDenomi_dVg *= T9;
        dDenomi_dVd *= T9;
        dDenomi_dVb *= T9;
    }
    const double ueff = Q(u0temp) / Denomi;
    T9 = -ueff / Denomi;
    const double dueff_dVg = T9 * dDenomi_dVg;
    const double dueff_dVd = T9 * dDenomi_dVd;
    const double dueff_dVb = T9 * dDenomi_dVb;

    /* saturation voltage Vdsat (b4ld.c:1614-1713) */
    const double vsattemp = Q(vsattemp);
    const double WVCox = Weff * vsattemp * coxe;
    const double WVCoxRds = WVCox * Rds;
    double Esat = 2.0 * vsattemp / ueff;
    double EsatL = Esat * Leff;
    T0 = -EsatL / ueff;
    double dEsatL_dVg = T0 * dueff_dVg;
    double dEsatL_dVd = T0 * dueff_dVd;
    double dEsatL_dVb = T0 * dueff_dVb;
    const double a1 = Q(a1), a2 = Q(a2);
    double Lambda, dLambda_dVg;
    if (a1 == 0.0) {
        Lambda = a2;
        dLambda_dVg = 0.0;
    } else if (a1 > 0.0) {
        T0 = 1.0 - a2;
        T1 = T0 - a1 * Vgsteff - 0.0001;
        T2 = sqrt(T1 * T1 + 0.0004 * T0);
        Lambda = a2 + T0 - 0.5 * (T1 + T2);
        dLambda_dVg = 0.5 * a1 * (1.0 + T1 / T2);
    } else {
        T1 = a2 + a1 * Vgsteff - 0.0001;
        T2 = sqrt(T1 * T1 + 0.0004 * a2);
        Lambda = 0.5 * (T1 + T2);
        dLambda_dVg = 0.5 * a1 * (1.0 + T1 / T2);
    }
    const double Vgst2Vtm = Vgsteff + 2.0 * Vtm;
    if (Rds > 0) {
        tmp2 = dRds_dVg / Rds + dWeff_dVg / Weff;
        tmp3 = dRds_dVb / Rds + dWeff_dVb / Weff;
    } else {
        tmp2 = dWeff_dVg / Weff;
        tmp3 = dWeff_dVb / Weff;
    }
    double Vdsat, dVdsat_dVg, dVdsat_dVd, dVdsat_dVb;
    if ((Rds == 0.0) && (Lambda == 1.0)) {
        T0 = 1.0 / (Abulk * EsatL + Vgst2Vtm);
        tmp1 = 0.0;
        T1 = T0 * T0;
        T2 = Vgst2Vtm * T0;
        T3 = EsatL * Vgst2Vtm;
        Vdsat = T3 * T0;
        const double dT0_dVg = -(Abulk * dEsatL_dVg + EsatL * dAbulk_dVg + 1.0) * T1;
        const double dT0_dVd = -(Abulk * dEsatL_dVd) * T1;
        const double dT0_dVb2 = -(Abulk * dEsatL_dVb + dAbulk_dVb * EsatL) * T1;
        dVdsat_dVg = T3 * dT0_dVg + T2 * dEsatL_dVg + EsatL * T0;
        dVdsat_dVd = T3 * dT0_dVd + T2 * dEsatL_dVd;
        dVdsat_dVb = T3 * dT0_dVb2 + T2 * dEsatL_dVb;
    } else {
        tmp1 = dLambda_dVg / (Lambda * Lambda);
        T9 = Abulk * WVCoxRds;
        T8 = Abulk * T9;
        T7 = Vgst2Vtm * T9;
        T6 = Vgst2Vtm * WVCoxRds;
        T0 = 2.0 * Abulk * (T9 - 1.0 + 1.0 / Lambda);
        const double dT0_dVg = 2.0 * (T8 * tmp2 - Abulk * tmp1 +
                                      (2.0 * T9 + 1.0 / Lambda - 1.0) * dAbulk_dVg);
        const double dT0_dVb2 = 2.0 * (T8 * (2.0 / Abulk * dAbulk_dVb + tmp3) +
                                       (1.0 / Lambda - 1.0) * dAbulk_dVb);
        const double dT0_dVd = 0.0;
        T1 = Vgst2Vtm * (2.0 / Lambda - 1.0) + Abulk * EsatL + 3.0 * T7;
        const double dT1_dVg = (2.0 / Lambda - 1.0) - 2.0 * Vgst2Vtm * tmp1 + Abulk * dEsatL_dVg +
                               EsatL * dAbulk_dVg + 3.0 * (T9 + T7 * tmp2 + T6 * dAbulk_dVg);
        const double dT1_dVb2 = Abulk * dEsatL_dVb + EsatL * dAbulk_dVb +
                                3.0 * (T6 * dAbulk_dVb + T7 * tmp3);
        const double dT1_dVd = Abulk * dEsatL_dVd;
        T2 = Vgst2Vtm * (EsatL + 2.0 * T6);
        const double dT2_dVg = EsatL + Vgst2Vtm * dEsatL_dVg + T6 * (4.0 + 2.0 * Vgst2Vtm * tmp2);
        const double dT2_dVb2 = Vgst2Vtm * (dEsatL_dVb + 2.0 * T6 * tmp3);
        const double dT2_dVd = Vgst2Vtm * dEsatL_dVd;
        T3 = sqrt(T1 * T1 - 2.0 * T0 * T2);
        Vdsat = (T1 - T3) / T0;
        dVdsat_dVg = (dT1_dVg - (T1 * dT1_dVg - dT0_dVg * T2 - T0 * dT2_dVg) / T3 -
                      Vdsat * dT0_dVg) / T0;
        dVdsat_dVb = (dT1_dVb2 - (T1 * dT1_dVb2 - dT0_dVb2 * T2 - T0 * dT2_dVb2) / T3 -
                      Vdsat * dT0_dVb2) / T0;
        dVdsat_dVd = (dT1_dVd - (T1 * dT1_dVd - T0 * dT2_dVd) / T3) / T0;
        (void)dT0_dVd;
    }

    /* effective drain voltage Vdseff (b4ld.c:1716-1755) */
    double Vdseff, dVdseff_dVg, dVdseff_dVd, dVdseff_dVb;
    {
        const double delta = Q(delta);
        T1 = Vdsat - Vds - delta;
        const double dT1_dVg = dVdsat_dVg;
        const double dT1_dVd = dVdsat_dVd - 1.0;
        const double dT1_dVb2 = dVdsat_dVb;
        T2 = sqrt(T1 * T1 + 4.0 * delta * Vdsat);
        T0 = T1 / T2;
        T9 = 2.0 * delta;
        T3 = T9 / T2;
        const double dT2_dVg = T0 * dT1_dVg + T3 * dVdsat_dVg;
        const double dT2_dVd = T0 * dT1_dVd + T3 * dVdsat_dVd;
        const double dT2_dVb2 = T0 * dT1_dVb2 + T3 * dVdsat_dVb;
        if (T1 >= 0.0) {
            Vdseff = Vdsat - 0.5 * (T1 + T2);
            dVdseff_dVg = dVdsat_dVg - 0.5 * (dT1_dVg + dT2_dVg);
            dVdseff_dVd = dVdsat_dVd - 0.5 * (dT1_dVd + dT2_dVd);
            dVdseff_dVb = dVdsat_dVb - 0.5 * (dT1_dVb2 + dT2_dVb2);
        } else {
            T4 = T9 / (T2 - T1);
            T5 = 1.0 - T4;
            T6 = Vdsat * T4 / (T2 - T1);
            Vdseff = Vdsat * T5;
            dVdseff_dVg = dVdsat_dVg * T5 + T6 * (dT2_dVg - dT1_dVg);
            dVdseff_dVd = dVdsat_dVd * T5 + T6 * (dT2_dVd - dT1_dVd);
            dVdseff_dVb = dVdsat_dVb * T5 + T6 * (dT2_dVb2 - dT1_dVb2);
        }
        if (Vds == 0.0) {
            Vdseff = 0.0;
            dVdseff_dVg = 0.0;
            dVdseff_dVb = 0.0;
        }
        if (Vdseff > Vds)
            Vdseff = Vds;
    }
    const double diffVds = Vds - Vdseff;

    /* Vasat (b4ld.c:1800-1822) */
    double Vasat, dVasat_dVg, dVasat_dVb, dVasat_dVd;
    {
        tmp4 = 1.0 - 0.5 * Abulk * Vdsat / Vgst2Vtm;
        T9 = WVCoxRds * Vgsteff;
        T8 = T9 / Vgst2Vtm;
        T0 = EsatL + Vdsat + 2.0 * T9 * tmp4;
        T7 = 2.0 * WVCoxRds * tmp4;
        const double dT0_dVg = dEsatL_dVg + dVdsat_dVg + T7 * (1.0 + tmp2 * Vgsteff) -
                               T8 * (Abulk * dVdsat_dVg - Abulk * Vdsat / Vgst2Vtm +
                                     Vdsat * dAbulk_dVg);
        const double dT0_dVb2 = dEsatL_dVb + dVdsat_dVb + T7 * tmp3 * Vgsteff -
                                T8 * (dAbulk_dVb * Vdsat + Abulk * dVdsat_dVb);
        const double dT0_dVd = dEsatL_dVd + dVdsat_dVd - T8 * Abulk * dVdsat_dVd;
        T9 = WVCoxRds * Abulk;
        T1 = 2.0 / Lambda - 1.0 + T9;
        const double dT1_dVg = -2.0 * tmp1 + WVCoxRds * (Abulk * tmp2 + dAbulk_dVg);
        const double dT1_dVb2 = dAbulk_dVb * WVCoxRds + T9 * tmp3;
        Vasat = T0 / T1;
        dVasat_dVg = (dT0_dVg - Vasat * dT1_dVg) / T1;
        dVasat_dVb = (dT0_dVb2 - Vasat * dT1_dVb2) / T1;
        dVasat_dVd = dT0_dVd / T1;
    }

    /* linear-region current Idl (b4ld.c:1824-1880) */
    double Idl, dIdl_dVg, dIdl_dVd, dIdl_dVb, Coxeff, beta, CoxeffWovL;
    double dbeta_dVg, dbeta_dVd, dbeta_dVb, gche;
    {
        tmp1 = Q(vtfbphi2);
        tmp2 = 2.0e8 * Q(toxp);
        const double dT0_dVg = 1.0 / tmp2;
        T0 = (Vgsteff + tmp1) * dT0_dVg;
        tmp3 = exp(Q(bdos) * 0.7 * log(T0));
        T1 = 1.0 + tmp3;
        T2 = Q(bdos) * 0.7 * tmp3 / T0;
        const double Tcen = Q(ados) * 1.9e-9 / T1;
        const double dTcen_dVg = -Tcen * T2 * dT0_dVg / T1;
        const double coxp = Q(coxp);
        Coxeff = epssub * coxp / (epssub + coxp * Tcen);
        const double dCoxeff_dVg = -Coxeff * Coxeff * dTcen_dVg / epssub;
        CoxeffWovL = Coxeff * Weff / Leff;
        beta = ueff * CoxeffWovL;
        T3 = ueff / Leff;
        dbeta_dVg = CoxeffWovL * dueff_dVg + T3 * (Weff * dCoxeff_dVg + Coxeff * dWeff_dVg);
        dbeta_dVd = CoxeffWovL * dueff_dVd;
        dbeta_dVb = CoxeffWovL * dueff_dVb + T3 * Coxeff * dWeff_dVb;
        const double AbovVgst2Vtm = Abulk / Vgst2Vtm;
        T0 = 1.0 - 0.5 * Vdseff * AbovVgst2Vtm;
        const double dT0_dVg2 = -0.5 * (Abulk * dVdseff_dVg - Abulk * Vdseff / Vgst2Vtm +
                                        Vdseff * dAbulk_dVg) / Vgst2Vtm;
        const double dT0_dVd = -0.5 * Abulk * dVdseff_dVd / Vgst2Vtm;
        const double dT0_dVb2 = -0.5 * (Abulk * dVdseff_dVb + dAbulk_dVb * Vdseff) / Vgst2Vtm;
        const double fgche1 = Vgsteff * T0;
        const double dfgche1_dVg = Vgsteff * dT0_dVg2 + T0;
        const double dfgche1_dVd = Vgsteff * dT0_dVd;
        const double dfgche1_dVb = Vgsteff * dT0_dVb2;
        T9 = Vdseff / EsatL;
        const double fgche2 = 1.0 + T9;
        const double dfgche2_dVg = (dVdseff_dVg - T9 * dEsatL_dVg) / EsatL;
        const double dfgche2_dVd = (dVdseff_dVd - T9 * dEsatL_dVd) / EsatL;
        const double dfgche2_dVb = (dVdseff_dVb - T9 * dEsatL_dVb) / EsatL;
        gche = beta * fgche1 / fgche2;
        const double dgche_dVg = (beta * dfgche1_dVg + fgche1 * dbeta_dVg - gche * dfgche2_dVg) / fgche2;
        const double dgche_dVd = (beta * dfgche1_dVd + fgche1 * dbeta_dVd - gche * dfgche2_dVd) / fgche2;
        const double dgche_dVb = (beta * dfgche1_dVb + fgche1 * dbeta_dVb - gche * dfgche2_dVb) / fgche2;
        T0 = 1.0 + gche * Rds;
        Idl = gche / T0;
        T1 = (1.0 - Idl * Rds) / T0;
        T2 = Idl * Idl;
        dIdl_dVg = T1 * dgche_dVg - T2 * dRds_dVg;
        dIdl_dVd = T1 * dgche_dVd;
        dIdl_dVb = T1 * dgche_dVb - T2 * dRds_dVb;
    }

    /* output-resistance terms FP, PvagTerm, VACLM, VADIBL, VADITS, VASCBE
     * (b4ld.c:1882-2046) */
    double FP, dFP_dVg;
    if (Q(fprout) <= 0.0) {
        FP = 1.0;
        dFP_dVg = 0.0;
    } else {
        T9 = Q(fprout) * sqrt(Leff) / Vgst2Vtm;
        FP = 1.0 / (1.0 + T9);
        dFP_dVg = FP * FP * T9 / Vgst2Vtm;
    }
    double PvagTerm, dPvagTerm_dVg, dPvagTerm_dVb, dPvagTerm_dVd;
    T8 = Q(pvag) / EsatL;
    T9 = T8 * Vgsteff;
    if (T9 > -0.9) {
        PvagTerm = 1.0 + T9;
        dPvagTerm_dVg = T8 * (1.0 - Vgsteff * dEsatL_dVg / EsatL);
        dPvagTerm_dVb = -T9 * dEsatL_dVb / EsatL;
        dPvagTerm_dVd = -T9 * dEsatL_dVd / EsatL;
    } else {
        T4 = 1.0 / (17.0 + 20.0 * T9);
        PvagTerm = (0.8 + T9) * T4;
        T4 *= T4;
        dPvagTerm_dVg = T8 * (1.0 - Vgsteff * dEsatL_dVg / EsatL) * T4;
        T9 *= T4 / EsatL;
        dPvagTerm_dVb = -T9 * dEsatL_dVb;
        dPvagTerm_dVd = -T9 * dEsatL_dVd;
    }
    const double litl = Q(litl), pclm = Q(pclm);
    double VACLM, Cclm, dVACLM_dVg, dVACLM_dVb, dVACLM_dVd, dCclm_dVg, dCclm_dVb, dCclm_dVd;
    if ((pclm > B4_MIN_EXP) && (diffVds > 1.0e-10)) {
        T0 = 1.0 + Rds * Idl;
        const double dT0_dVg = dRds_dVg * Idl + Rds * dIdl_dVg;
        const double dT0_dVd = Rds * dIdl_dVd;
        const double dT0_dVb2 = dRds_dVb * Idl + Rds * dIdl_dVb;
        T2 = Vdsat / Esat;
        T1 = Leff + T2;
        const double dT1_dVg = (dVdsat_dVg - T2 * dEsatL_dVg / Leff) / Esat;
        const double dT1_dVd = (dVdsat_dVd - T2 * dEsatL_dVd / Leff) / Esat;
        const double dT1_dVb2 = (dVdsat_dVb - T2 * dEsatL_dVb / Leff) / Esat;
        Cclm = FP * PvagTerm * T0 * T1 / (pclm * litl);
        dCclm_dVg = Cclm * (dFP_dVg / FP + dPvagTerm_dVg / PvagTerm + dT0_dVg / T0 + dT1_dVg / T1);
        dCclm_dVb = Cclm * (dPvagTerm_dVb / PvagTerm + dT0_dVb2 / T0 + dT1_dVb2 / T1);
        dCclm_dVd = Cclm * (dPvagTerm_dVd / PvagTerm + dT0_dVd / T0 + dT1_dVd / T1);
        VACLM = Cclm * diffVds;
        dVACLM_dVg = dCclm_dVg * diffVds - dVdseff_dVg * Cclm;
        dVACLM_dVb = dCclm_dVb * diffVds - dVdseff_dVb * Cclm;
        dVACLM_dVd = dCclm_dVd * diffVds + (1.0 - dVdseff_dVd) * Cclm;
    } else {
        VACLM = Cclm = B4_MAX_EXP;
        dVACLM_dVd = dVACLM_dVg = dVACLM_dVb = 0.0;
        dCclm_dVd = dCclm_dVg = dCclm_dVb = 0.0;
    }
    double VADIBL, dVADIBL_dVg, dVADIBL_dVb, dVADIBL_dVd;
    if (Q(thetaRout) > B4_MIN_EXP) {
        T8 = Abulk * Vdsat;
        T0 = Vgst2Vtm * T8;
        const double dT0_dVg = Vgst2Vtm * Abulk * dVdsat_dVg + T8 + Vgst2Vtm * Vdsat * dAbulk_dVg;
        const double dT0_dVb2 = Vgst2Vtm * (dAbulk_dVb * Vdsat + Abulk * dVdsat_dVb);
        const double dT0_dVd = Vgst2Vtm * Abulk * dVdsat_dVd;
        T1 = Vgst2Vtm + T8;
        const double dT1_dVg = 1.0 + Abulk * dVdsat_dVg + Vdsat * dAbulk_dVg;
        const double dT1_dVb2 = Abulk * dVdsat_dVb + dAbulk_dVb * Vdsat;
        const double dT1_dVd = Abulk * dVdsat_dVd;
        T9 = T1 * T1;
        T2 = Q(thetaRout);
        VADIBL = (Vgst2Vtm - T0 / T1) / T2;
        dVADIBL_dVg = (1.0 - dT0_dVg / T1 + T0 * dT1_dVg / T9) / T2;
        dVADIBL_dVb = (-dT0_dVb2 / T1 + T0 * dT1_dVb2 / T9) / T2;
        dVADIBL_dVd = (-dT0_dVd / T1 + T0 * dT1_dVd / T9) / T2;
        const double pdiblb = Q(pdiblb);
        T7 = pdiblb * Vbseff;
        if (T7 >= -0.9) {
            T3 = 1.0 / (1.0 + T7);
            VADIBL *= T3;
            dVADIBL_dVg *= T3;
            dVADIBL_dVb = (dVADIBL_dVb - VADIBL * pdiblb) * T3;
            dVADIBL_dVd *= T3;
        } else {
            T4 = 1.0 / (0.8 + T7);
            T3 = (17.0 + 20.0 * T7) * T4;
            dVADIBL_dVg *= T3;
            dVADIBL_dVb = dVADIBL_dVb * T3 - VADIBL * pdiblb * T4 * T4;
            dVADIBL_dVd *= T3;
            VADIBL *= T3;
        }
        dVADIBL_dVg = dVADIBL_dVg * PvagTerm + VADIBL * dPvagTerm_dVg;
        dVADIBL_dVb = dVADIBL_dVb * PvagTerm + VADIBL * dPvagTerm_dVb;
        dVADIBL_dVd = dVADIBL_dVd * PvagTerm + VADIBL * dPvagTerm_dVd;
        VADIBL *= PvagTerm;
    } else {
        VADIBL = B4_MAX_EXP;
        dVADIBL_dVd = dVADIBL_dVg = dVADIBL_dVb = 0.0;
    }
    const double Va = Vasat + VACLM;
    const double dVa_dVg = dVasat_dVg + dVACLM_dVg;
    const double dVa_dVb = dVasat_dVb + dVACLM_dVb;
    const double dVa_dVd = dVasat_dVd + dVACLM_dVd;
    double VADITS, dVADITS_dVg, dVADITS_dVd;
    {
        double dT1_dVd;
        T0 = Q(pditsd) * Vds;
        if (T0 > B4_EXP_THRESHOLD) {
            T1 = B4_MAX_EXP;
            dT1_dVd = 0;
        } else {
            T1 = exp(T0);
            dT1_dVd = T1 * Q(pditsd);
        }
        if (Q(pdits) > B4_MIN_EXP) {
            T2 = 1.0 + Q(pditsl) * Leff;
            VADITS = (1.0 + T2 * T1) / Q(pdits);
            dVADITS_dVg = VADITS * dFP_dVg;
            dVADITS_dVd = FP * T2 * dT1_dVd / Q(pdits);
            VADITS *= FP;
        } else {
            VADITS = B4_MAX_EXP;
            dVADITS_dVg = dVADITS_dVd = 0;
        }
    }
    double VASCBE, dVASCBE_dVg, dVASCBE_dVd, dVASCBE_dVb;
    {
        const double pscbe1 = Q(pscbe1), pscbe2 = Q(pscbe2);
        if ((pscbe2 > 0.0) && (pscbe1 >= 0.0)) {
            if (diffVds > pscbe1 * litl / B4_EXP_THRESHOLD) {
                T0 = pscbe1 * litl / diffVds;
                VASCBE = Leff * exp(T0) / pscbe2;
                T1 = T0 * VASCBE / diffVds;
                dVASCBE_dVg = T1 * dVdseff_dVg;
                dVASCBE_dVd = -T1 * (1.0 - dVdseff_dVd);
                dVASCBE_dVb = T1 * dVdseff_dVb;
            } else {
                VASCBE = B4_MAX_EXP * Leff / pscbe2;
                dVASCBE_dVg = dVASCBE_dVd = dVASCBE_dVb = 0.0;
            }
        } else {
            VASCBE = B4_MAX_EXP;
            dVASCBE_dVg = dVASCBE_dVd = dVASCBE_dVb = 0.0;
        }
    }

    /* drain current with DIBL, DITS, CLM, substrate current and SCBE
     * (b4ld.c:2048-2146) */
    double Idsa, dIdsa_dVg, dIdsa_dVd, dIdsa_dVb;
    T9 = diffVds / VADIBL;
    T0 = 1.0 + T9;
    Idsa = Idl * T0;
    dIdsa_dVg = T0 * dIdl_dVg - Idl * (dVdseff_dVg + T9 * dVADIBL_dVg) / VADIBL;
    dIdsa_dVd = T0 * dIdl_dVd + Idl * (1.0 - dVdseff_dVd - T9 * dVADIBL_dVd) / VADIBL;
    dIdsa_dVb = T0 * dIdl_dVb - Idl * (dVdseff_dVb + T9 * dVADIBL_dVb) / VADIBL;
    T9 = diffVds / VADITS;
    T0 = 1.0 + T9;
    dIdsa_dVg = T0 * dIdsa_dVg - Idsa * (dVdseff_dVg + T9 * dVADITS_dVg) / VADITS;
    dIdsa_dVd = T0 * dIdsa_dVd + Idsa * (1.0 - dVdseff_dVd - T9 * dVADITS_dVd) / VADITS;
    dIdsa_dVb = T0 * dIdsa_dVb - Idsa * dVdseff_dVb / VADITS;
    Idsa *= T0;
    {
        T0 = log(Va / Vasat);
        const double dT0_dVg = dVa_dVg / Va - dVasat_dVg / Vasat;
        const double dT0_dVb2 = dVa_dVb / Va - dVasat_dVb / Vasat;
        const double dT0_dVd = dVa_dVd / Va - dVasat_dVd / Vasat;
        T1 = T0 / Cclm;
        T9 = 1.0 + T1;
        const double dT9_dVg2 = (dT0_dVg - T1 * dCclm_dVg) / Cclm;
        const double dT9_dVb2 = (dT0_dVb2 - T1 * dCclm_dVb) / Cclm;
        const double dT9_dVd2 = (dT0_dVd - T1 * dCclm_dVd) / Cclm;
        dIdsa_dVg = dIdsa_dVg * T9 + Idsa * dT9_dVg2;
        dIdsa_dVb = dIdsa_dVb * T9 + Idsa * dT9_dVb2;
        dIdsa_dVd = dIdsa_dVd * T9 + Idsa * dT9_dVd2;
        Idsa *= T9;
    }
    double Isub, Gbd, Gbb, Gbg;
    {
        const double tmp = Q(alpha0) + Q(alpha1) * Leff;
        const double beta0 = Q(beta0);
        if ((tmp <= 0.0) || (beta0 <= 0.0)) {
            Isub = Gbd = Gbb = Gbg = 0.0;
        } else {
            double dT1_dVg, dT1_dVd;
            T2 = tmp / Leff;
            if (diffVds > beta0 / B4_EXP_THRESHOLD) {
                T0 = -beta0 / diffVds;
                T1 = T2 * diffVds * exp(T0);
                T3 = T1 / diffVds * (T0 - 1.0);
                dT1_dVg = T3 * dVdseff_dVg;
                dT1_dVd = T3 * (dVdseff_dVd - 1.0);
                dT1_dVb = T3 * dVdseff_dVb;
            } else {
                T3 = T2 * B4_MIN_EXP;
                T1 = T3 * diffVds;
                dT1_dVg = -T3 * dVdseff_dVg;
                dT1_dVd = T3 * (1.0 - dVdseff_dVd);
                dT1_dVb = -T3 * dVdseff_dVb;
            }
            T4 = Idsa * Vdseff;
            Isub = T1 * T4;
            Gbg = T1 * (dIdsa_dVg * Vdseff + Idsa * dVdseff_dVg) + T4 * dT1_dVg;
            Gbd = T1 * (dIdsa_dVd * Vdseff + Idsa * dVdseff_dVd) + T4 * dT1_dVd;
            Gbb = T1 * (dIdsa_dVb * Vdseff + Idsa * dVdseff_dVb) + T4 * dT1_dVb;
            Gbd += Gbg * dVgsteff_dVd;
            Gbb += Gbg * dVgsteff_dVb;
            Gbg *= dVgsteff_dVg;
            Gbb *= dVbseff_dVb;
        }
    }
    double csub = Isub, gbbs = Gbb, gbgs = Gbg, gbds = Gbd;
    T9 = diffVds / VASCBE;
    T0 = 1.0 + T9;
    const double Ids = Idsa * T0;
    double Gm = T0 * dIdsa_dVg - Idsa * (dVdseff_dVg + T9 * dVASCBE_dVg) / VASCBE;
    double Gds = T0 * dIdsa_dVd + Idsa * (1.0 - dVdseff_dVd - T9 * dVASCBE_dVd) / VASCBE;
    double Gmb = T0 * dIdsa_dVb - Idsa * (dVdseff_dVb + T9 * dVASCBE_dVb) / VASCBE;
    tmp1 = Gds + Gm * dVgsteff_dVd;
    tmp2 = Gmb + Gm * dVgsteff_dVb;
    tmp3 = Gm;
    Gm = (Ids * dVdseff_dVg + Vdseff * tmp3) * dVgsteff_dVg;
    Gds = Ids * (dVdseff_dVd + dVdseff_dVg * dVgsteff_dVd) + Vdseff * tmp1;
    Gmb = (Ids * (dVdseff_dVb + dVdseff_dVg * dVgsteff_dVb) + Vdseff * tmp2) * dVbseff_dVb;
    double cdrain = Ids * Vdseff;
    double gds = Gds, gm = Gm, gmbs = Gmb;

    /* GIDL / GISL, gidlMod 0 (b4ld.c:2305-2384) */
    double Igidl, Ggidld, Ggidlg, Ggidlb, Igisl, Ggisls, Ggislg, Ggislb;
    {
        const double T0g = 3.0 * toxe;
        const double weffCJ = Q(weffCJ);
        const double agidl = Q(agidl), bgidl = Q(bgidl), cgidl = Q(cgidl);
        T1 = (vds - vgs_eff - Q(egidl)) / T0g;
        if ((agidl <= 0.0) || (bgidl <= 0.0) || (T1 <= 0.0) || (cgidl <= 0.0) || (vbd > 0.0)) {
            Igidl = Ggidld = Ggidlg = Ggidlb = 0.0;
        } else {
            const double dT1_dVd = 1.0 / T0g;
            const double dT1_dVg = -dvgs_eff_dvg * dT1_dVd;
            T2 = bgidl / T1;
            if (T2 < 100.0) {
                Igidl = agidl * weffCJ * T1 * exp(-T2);
                T3 = Igidl * (1.0 + T2) / T1;
                Ggidld = T3 * dT1_dVd;
                Ggidlg = T3 * dT1_dVg;
            } else {
                Igidl = agidl * weffCJ * 3.720075976e-44;
                Ggidld = Igidl * dT1_dVd;
                Ggidlg = Igidl * dT1_dVg;
                Igidl *= T1;
            }
            T4 = vbd * vbd;
            T5 = -vbd * T4;
            T6 = cgidl + T5;
            T7 = T5 / T6;
            T8 = 3.0 * cgidl * T4 / T6 / T6;
            Ggidld = Ggidld * T7 + Igidl * T8;
            Ggidlg = Ggidlg * T7;
            Ggidlb = -Igidl * T8;
            Igidl *= T7;
        }
        const double agisl = Q(agisl), bgisl = Q(bgisl), cgisl = Q(cgisl);
        T1 = (-vds - vgd_eff - Q(egisl)) / T0g;
        if ((agisl <= 0.0) || (bgisl <= 0.0) || (T1 <= 0.0) || (cgisl <= 0.0) || (vbs > 0.0)) {
            Igisl = Ggisls = Ggislg = Ggislb = 0.0;
        } else {
            const double dT1_dVd = 1.0 / T0g;
            const double dT1_dVg = -dvgd_eff_dvg * dT1_dVd;
            T2 = bgisl / T1;
            if (T2 < 100.0) {
                Igisl = agisl * weffCJ * T1 * exp(-T2);
                T3 = Igisl * (1.0 + T2) / T1;
                Ggisls = T3 * dT1_dVd;
                Ggislg = T3 * dT1_dVg;
            } else {
                Igisl = agisl * weffCJ * 3.720075976e-44;
                Ggisls = Igisl * dT1_dVd;
                Ggislg = Igisl * dT1_dVg;
                Igisl *= T1;
            }
            T4 = vbs * vbs;
            T5 = -vbs * T4;
            T6 = cgisl + T5;
            T7 = T5 / T6;
            T8 = 3.0 * cgisl * T4 / T6 / T6;
            Ggisls = Ggisls * T7 + Igisl * T8;
            Ggislg = Ggislg * T7;
            Ggislb = -Igisl * T8;
            Igisl *= T7;
        }
    }

    /* multi-finger scaling (b4ld.c:2921-2958) */
    const double nf = Q(nf);
    if (nf != 1.0) {
        cdrain *= nf;
        gds *= nf;
        gm *= nf;
        gmbs *= nf;
        gbbs *= nf;
        gbgs *= nf;
        gbds *= nf;
        csub *= nf;
        Igidl *= nf;
        Ggidld *= nf;
        Ggidlg *= nf;
        Ggidlb *= nf;
        Igisl *= nf;
        Ggisls *= nf;
        Ggislg *= nf;
        Ggislb *= nf;
    }
    (void)Ggidlb;

    /* ---- C-V, capMod 2 charge-thickness model (b4ld.c:3014-3945) ---- */
    double qgate = 0.0, qdrn = 0.0, qbulk = 0.0;
    double cggb = 0, cgsb = 0, cgdb = 0, cdgb = 0, cdsb = 0, cddb = 0, cbgb = 0, cbsb = 0, cbdb = 0;
    if ((Q(xpart) < 0) || (!ccn)) {
        /* charges and capacitances stay zero */
    } else {
        double VbseffCV, dVbseffCV_dVb;
        if (Vbseff < 0.0) {
            VbseffCV = Vbseff;
            dVbseffCV_dVb = 1.0;
        } else {
            VbseffCV = phi - Phis;
            dVbseffCV_dVb = -dPhis_dVb;
        }
        const double CoxWL = coxe * Q(weffCV) * Q(leffCV) * nf;
        (void)CoxWL;
        /* VgsteffCV, cvchargeMod 0 (b4ld.c:3351-3387) */
        {
            const double noff = n_ * Q(noff);
            const double dnoff_dVd = Q(noff) * dn_dVd;
            const double dnoff_dVb = Q(noff) * dn_dVb;
            T0 = Vtm * noff;
            const double voffcv = Q(voffcv);
            const double VgstNVt = (Vgst - voffcv) / T0;
            if (VgstNVt > B4_EXP_THRESHOLD) {
                Vgsteff = Vgst - voffcv;
                dVgsteff_dVg = dVgs_eff_dVg;
                dVgsteff_dVd = -dVth_dVd;
                dVgsteff_dVb = -dVth_dVb;
            } else if (VgstNVt < -B4_EXP_THRESHOLD) {
                Vgsteff = T0 * log(1.0 + B4_MIN_EXP);
                dVgsteff_dVg = 0.0;
                dVgsteff_dVd = Vgsteff / noff;
                dVgsteff_dVb = dVgsteff_dVd * dnoff_dVb;
                dVgsteff_dVd *= dnoff_dVd;
            } else {
                ExpVgst = exp(VgstNVt);
                Vgsteff = T0 * log(1.0 + ExpVgst);
                dVgsteff_dVg = ExpVgst / (1.0 + ExpVgst);
                dVgsteff_dVd = -dVgsteff_dVg * (dVth_dVd + (Vgst - voffcv) / noff * dnoff_dVd) +
                               Vgsteff / noff * dnoff_dVd;
                dVgsteff_dVb = -dVgsteff_dVg * (dVth_dVb + (Vgst - voffcv) / noff * dnoff_dVb) +
                               Vgsteff / noff * dnoff_dVb;
                dVgsteff_dVg *= dVgs_eff_dVg;
            }
        }
        /* charge-thickness model (b4ld.c:3632-3945) */
        const double vfbzb = Q(vfbzb);
        double V3 = vfbzb - Vgs_eff + VbseffCV - B4_DELTA_3;
        if (vfbzb <= 0.0)
            T0 = sqrt(V3 * V3 - 4.0 * B4_DELTA_3 * vfbzb);
        else
            T0 = sqrt(V3 * V3 + 4.0 * B4_DELTA_3 * vfbzb);
        T1 = 0.5 * (1.0 + V3 / T0);
        const double Vfbeff = vfbzb - 0.5 * (V3 + T0);
        const double dVfbeff_dVg = T1 * dVgs_eff_dVg;
        const double dVfbeff_dVb = -T1 * dVbseffCV_dVb;
        const double Cox = Q(coxp);
        double Tox = 1.0e8 * Q(toxp);
        T0 = (Vgs_eff - VbseffCV - vfbzb) / Tox;
        const double dT0_dVg = dVgs_eff_dVg / Tox;
        const double dT0_dVb2 = -dVbseffCV_dVb / Tox;
        const double acde = Q(acde), ldeb = Q(ldeb);
        double tmp = T0 * acde;
        double Tcen, dTcen_dVg, dTcen_dVb, dTcen_dVd;
        if ((-B4_EXP_THRESHOLD < tmp) && (tmp < B4_EXP_THRESHOLD)) {
            Tcen = ldeb * exp(tmp);
            dTcen_dVg = acde * Tcen;
            dTcen_dVb = dTcen_dVg * dT0_dVb2;
            dTcen_dVg *= dT0_dVg;
        } else if (tmp <= -B4_EXP_THRESHOLD) {
            Tcen = ldeb * B4_MIN_EXP;
            dTcen_dVg = dTcen_dVb = 0.0;
        } else {
            Tcen = ldeb * B4_MAX_EXP;
            dTcen_dVg = dTcen_dVb = 0.0;
        }
        const double LINK = 1.0e-3 * Q(toxp);
        V3 = ldeb - Tcen - LINK;
        const double V4 = sqrt(V3 * V3 + 4.0 * LINK * ldeb);
        Tcen = ldeb - 0.5 * (V3 + V4);
        T1 = 0.5 * (1.0 + V3 / V4);
        dTcen_dVg *= T1;
        dTcen_dVb *= T1;
        double Ccen = epssub / Tcen;
        T2 = Cox / (Cox + Ccen);
        double Coxeff2 = T2 * Ccen;
        T3 = -Ccen / Tcen;
        double dCoxeff_dVg = T2 * T2 * T3;
        double dCoxeff_dVb = dCoxeff_dVg * dTcen_dVb;
        dCoxeff_dVg *= dTcen_dVg;
        const double CoxWLb = coxe * Q(weffCV) * Q(leffCV) * nf;
        double CoxWLcen = CoxWLb * Coxeff2 / coxe;
        const double Qac0 = CoxWLcen * (Vfbeff - vfbzb);
        double QovCox = Qac0 / Coxeff2;
        const double dQac0_dVg = CoxWLcen * dVfbeff_dVg + QovCox * dCoxeff_dVg;
        const double dQac0_dVb = CoxWLcen * dVfbeff_dVb + QovCox * dCoxeff_dVb;
        T0 = 0.5 * k1ox;
        T3 = Vgs_eff - Vfbeff - VbseffCV - Vgsteff;
        if (k1ox == 0.0) {
            T1 = 0.0;
            T2 = 0.0;
        } else if (T3 < 0.0) {
            T1 = T0 + T3 / k1ox;
            T2 = CoxWLcen;
        } else {
            T1 = sqrt(T0 * T0 + T3);
            T2 = CoxWLcen * T0 / T1;
        }
        const double Qsub0 = CoxWLcen * k1ox * (T1 - T0);
        QovCox = Qsub0 / Coxeff2;
        const double dQsub0_dVg = T2 * (dVgs_eff_dVg - dVfbeff_dVg - dVgsteff_dVg) + QovCox * dCoxeff_dVg;
        const double dQsub0_dVd = -T2 * dVgsteff_dVd;
        const double dQsub0_dVb = -T2 * (dVfbeff_dVb + dVbseffCV_dVb + dVgsteff_dVb) + QovCox * dCoxeff_dVb;
        double Denomi2;
        if (k1ox <= 0.0) {
            Denomi2 = 0.25 * Q(moin) * Vtm;
            T0 = 0.5 * sqrtPhi;
        } else {
            Denomi2 = Q(moin) * Vtm * k1ox * k1ox;
            T0 = k1ox * sqrtPhi;
        }
        T1 = 2.0 * T0 + Vgsteff;
        const double DeltaPhi = Vtm * log(1.0 + T1 * Vgsteff / Denomi2);
        const double dDeltaPhi_dVg = 2.0 * Vtm * (T1 - T0) / (Denomi2 + T1 * Vgsteff);
        T0 = Vgsteff - DeltaPhi - 0.001;
        const double dT0_dVg3 = 1.0 - dDeltaPhi_dVg;
        T1 = sqrt(T0 * T0 + Vgsteff * 0.004);
        const double VgDP = 0.5 * (T0 + T1);
        const double dVgDP_dVg = 0.5 * (dT0_dVg3 + (T0 * dT0_dVg3 + 0.002) / T1);
        Tox += Tox;
        T0 = (Vgsteff + Q(vtfbphi2)) / Tox;
        tmp = exp(Q(bdos) * 0.7 * log(T0));
        T1 = 1.0 + tmp;
        T2 = Q(bdos) * 0.7 * tmp / (T0 * Tox);
        Tcen = Q(ados) * 1.9e-9 / T1;
        dTcen_dVg = -Tcen * T2 / T1;
        dTcen_dVd = dTcen_dVg * dVgsteff_dVd;
        dTcen_dVb = dTcen_dVg * dVgsteff_dVb;
        dTcen_dVg *= dVgsteff_dVg;
        Ccen = epssub / Tcen;
        T0 = Cox / (Cox + Ccen);
        Coxeff2 = T0 * Ccen;
        T1 = -Ccen / Tcen;
        dCoxeff_dVg = T0 * T0 * T1;
        const double dCoxeff_dVd = dCoxeff_dVg * dTcen_dVd;
        dCoxeff_dVb = dCoxeff_dVg * dTcen_dVb;
        dCoxeff_dVg *= dTcen_dVg;
        CoxWLcen = CoxWLb * Coxeff2 / coxe;
        const double AbulkCV = Abulk0_Q * Q(abulkCVfactor);
        const double dAbulkCV_dVb = Q(abulkCVfactor) * dAbulk0_Q_dVb;
        const double VdsatCV = VgDP / AbulkCV;
        T0 = VdsatCV - Vds - B4_DELTA_4;
        const double dT0_dVg4 = dVgDP_dVg / AbulkCV;
        const double dT0_dVb4 = -VdsatCV * dAbulkCV_dVb / AbulkCV;
        T1 = sqrt(T0 * T0 + 4.0 * B4_DELTA_4 * VdsatCV);
        double dT1_dVg = (T0 + B4_DELTA_4 + B4_DELTA_4) / T1;
        const double dT1_dVd = -T0 / T1;
        const double dT1_dVb4 = dT1_dVg * dT0_dVb4;
        dT1_dVg *= dT0_dVg4;
        double VdseffCV, dVdseffCV_dVg, dVdseffCV_dVd, dVdseffCV_dVb;
        if (T0 >= 0.0) {
            VdseffCV = VdsatCV - 0.5 * (T0 + T1);
            dVdseffCV_dVg = 0.5 * (dT0_dVg4 - dT1_dVg);
            dVdseffCV_dVd = 0.5 * (1.0 - dT1_dVd);
            dVdseffCV_dVb = 0.5 * (dT0_dVb4 - dT1_dVb4);
        } else {
            T3 = (B4_DELTA_4 + B4_DELTA_4) / (T1 - T0);
            T4 = 1.0 - T3;
            T5 = VdsatCV * T3 / (T1 - T0);
            VdseffCV = VdsatCV * T4;
            dVdseffCV_dVg = dT0_dVg4 * T4 + T5 * (dT1_dVg - dT0_dVg4);
            dVdseffCV_dVd = T5 * (dT1_dVd + 1.0);
            dVdseffCV_dVb = dT0_dVb4 * (T4 - T5) + T5 * dT1_dVb4;
        }
        if (Vds == 0.0) {
            VdseffCV = 0.0;
            dVdseffCV_dVg = 0.0;
            dVdseffCV_dVb = 0.0;
        }
        T0 = AbulkCV * VdseffCV;
        T1 = VgDP;
        T2 = 12.0 * (T1 - 0.5 * T0 + 1.0e-20);
        T3 = T0 / T2;
        T4 = 1.0 - 12.0 * T3 * T3;
        T5 = AbulkCV * (6.0 * T0 * (4.0 * T1 - T0) / (T2 * T2) - 0.5);
        T6 = T5 * VdseffCV / AbulkCV;
        qgate = CoxWLcen * (T1 - T0 * (0.5 - T3));
        QovCox = qgate / Coxeff2;
        double Cgg1 = CoxWLcen * (T4 * dVgDP_dVg + T5 * dVdseffCV_dVg);
        const double Cgd1 = CoxWLcen * T5 * dVdseffCV_dVd + Cgg1 * dVgsteff_dVd + QovCox * dCoxeff_dVd;
        const double Cgb1 = CoxWLcen * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) +
                            Cgg1 * dVgsteff_dVb + QovCox * dCoxeff_dVb;
        Cgg1 = Cgg1 * dVgsteff_dVg + QovCox * dCoxeff_dVg;
        T7 = 1.0 - AbulkCV;
        T8 = T2 * T2;
        T9 = 12.0 * T7 * T0 * T0 / (T8 * AbulkCV);
        T10 = T9 * dVgDP_dVg;
        T11 = -T7 * T5 / AbulkCV;
        T12 = -(T9 * T1 / AbulkCV + VdseffCV * (0.5 - T0 / T2));
        qbulk = CoxWLcen * T7 * (0.5 * VdseffCV - T0 * VdseffCV / T2);
        QovCox = qbulk / Coxeff2;
        double Cbg1 = CoxWLcen * (T10 + T11 * dVdseffCV_dVg);
        const double Cbd1 = CoxWLcen * T11 * dVdseffCV_dVd + Cbg1 * dVgsteff_dVd + QovCox * dCoxeff_dVd;
        const double Cbb1 = CoxWLcen * (T11 * dVdseffCV_dVb + T12 * dAbulkCV_dVb) +
                            Cbg1 * dVgsteff_dVb + QovCox * dCoxeff_dVb;
        Cbg1 = Cbg1 * dVgsteff_dVg + QovCox * dCoxeff_dVg;
        double qsrc, Csg, Csd, Csb;
        const double xpart = Q(xpart);
        if (xpart > 0.5) {
            /* 0/100 partition */
            qsrc = -CoxWLcen * (T1 / 2.0 + T0 / 4.0 - 0.5 * T0 * T0 / T2);
            QovCox = qsrc / Coxeff2;
            T2 += T2;
            T3 = T2 * T2;
            T7 = -(0.25 - 12.0 * T0 * (4.0 * T1 - T0) / T3);
            T4 = -(0.5 + 24.0 * T0 * T0 / T3) * dVgDP_dVg;
            T5 = T7 * AbulkCV;
            T6 = T7 * VdseffCV;
            Csg = CoxWLcen * (T4 + T5 * dVdseffCV_dVg);
            Csd = CoxWLcen * T5 * dVdseffCV_dVd + Csg * dVgsteff_dVd + QovCox * dCoxeff_dVd;
            Csb = CoxWLcen * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Csg * dVgsteff_dVb +
                  QovCox * dCoxeff_dVb;
            Csg = Csg * dVgsteff_dVg + QovCox * dCoxeff_dVg;
        } else if (xpart < 0.5) {
            /* 40/60 partition */
            T2 = T2 / 12.0;
            T3 = 0.5 * CoxWLcen / (T2 * T2);
            T4 = T1 * (2.0 * T0 * T0 / 3.0 + T1 * (T1 - 4.0 * T0 / 3.0)) - 2.0 * T0 * T0 * T0 / 15.0;
            qsrc = -T3 * T4;
            QovCox = qsrc / Coxeff2;
            T8 = 4.0 / 3.0 * T1 * (T1 - T0) + 0.4 * T0 * T0;
            T5 = -2.0 * qsrc / T2 - T3 * (T1 * (3.0 * T1 - 8.0 * T0 / 3.0) + 2.0 * T0 * T0 / 3.0);
            T6 = AbulkCV * (qsrc / T2 + T3 * T8);
            T7 = T6 * VdseffCV / AbulkCV;
            Csg = T5 * dVgDP_dVg + T6 * dVdseffCV_dVg;
            Csd = Csg * dVgsteff_dVd + T6 * dVdseffCV_dVd + QovCox * dCoxeff_dVd;
            Csb = Csg * dVgsteff_dVb + T6 * dVdseffCV_dVb + T7 * dAbulkCV_dVb + QovCox * dCoxeff_dVb;
            Csg = Csg * dVgsteff_dVg + QovCox * dCoxeff_dVg;
        } else {
            /* 50/50 partition */
            qsrc = -0.5 * qgate;
            Csg = -0.5 * Cgg1;
            Csd = -0.5 * Cgd1;
            Csb = -0.5 * Cgb1;
        }
        qgate += Qac0 + Qsub0 - qbulk;
        qbulk -= (Qac0 + Qsub0);
        qdrn = -(qgate + qbulk + qsrc);
        const double Cbg = Cbg1 - dQac0_dVg - dQsub0_dVg;
        const double Cbd = Cbd1 - dQsub0_dVd;
        double Cbb = Cbb1 - dQac0_dVb - dQsub0_dVb;
        const double Cgg = Cgg1 - Cbg;
        const double Cgd = Cgd1 - Cbd;
        double Cgb = Cgb1 - Cbb;
        Cgb *= dVbseff_dVb;
        Cbb *= dVbseff_dVb;
        Csb *= dVbseff_dVb;
        cggb = Cgg;
        cgsb = -(Cgg + Cgd + Cgb);
        cgdb = Cgd;
        cdgb = -(Cgg + Cbg + Csg);
        cdsb = (Cgg + Cgd + Cgb + Cbg + Cbd + Cbb + Csg + Csd + Csb);
        cddb = -(Cgd + Cbd + Csd);
        cbgb = Cbg;
        cbsb = -(Cbg + Cbd + Cbb);
        cbdb = Cbd;
    }

    /* ---- junction capacitances (b4ld.c:3946-4058) ---- */
    double capbs = 0.0, capbd = 0.0;
    if (ccn) {
        const double czbd = Q(czbd), czbs = Q(czbs), czbdsw = Q(czbdsw), czbdswg = Q(czbdswg);
        const double czbssw = Q(czbssw), czbsswg = Q(czbsswg);
        const double MJS = Q(MJS), MJSWS = Q(MJSWS), MJSWGS = Q(MJSWGS);
        const double MJD = Q(MJD), MJSWD = Q(MJSWD), MJSWGD = Q(MJSWGD);
        double arg, sarg;
        if (vbs_jct == 0.0) {
            st0[B4S_QBS] = 0.0;
            capbs = czbs + czbssw + czbsswg;
        } else if (vbs_jct < 0.0) {
            if (czbs > 0.0) {
                arg = 1.0 - vbs_jct / Q(PhiBS);
                if (MJS == 0.5)
                    sarg = 1.0 / sqrt(arg);
                else
                    sarg = exp(-MJS * log(arg));
                st0[B4S_QBS] = Q(PhiBS) * czbs * (1.0 - arg * sarg) / (1.0 - MJS);
                capbs = czbs * sarg;
            } else {
                st0[B4S_QBS] = 0.0;
                capbs = 0.0;
            }
            if (czbssw > 0.0) {
                arg = 1.0 - vbs_jct / Q(PhiBSWS);
                if (MJSWS == 0.5)
                    sarg = 1.0 / sqrt(arg);
                else
                    sarg = exp(-MJSWS * log(arg));
                st0[B4S_QBS] += Q(PhiBSWS) * czbssw * (1.0 - arg * sarg) / (1.0 - MJSWS);
                capbs += czbssw * sarg;
            }
            if (czbsswg > 0.0) {
                arg = 1.0 - vbs_jct / Q(PhiBSWGS);
                if (MJSWGS == 0.5)
                    sarg = 1.0 / sqrt(arg);
                else
                    sarg = exp(-MJSWGS * log(arg));
                st0[B4S_QBS] += Q(PhiBSWGS) * czbsswg * (1.0 - arg * sarg) / (1.0 - MJSWGS);
                capbs += czbsswg * sarg;
            }
        } else {
            T0 = czbs + czbssw + czbsswg;
            T1 = vbs_jct * (czbs * MJS / Q(PhiBS) + czbssw * MJSWS / Q(PhiBSWS) +
                            czbsswg * MJSWGS / Q(PhiBSWGS));
            st0[B4S_QBS] = vbs_jct * (T0 + 0.5 * T1);
            capbs = T0 + T1;
        }
        if (vbd_jct == 0.0) {
            st0[B4S_QBD] = 0.0;
            capbd = czbd + czbdsw + czbdswg;
        } else if (vbd_jct < 0.0) {
            if (czbd > 0.0) {
                arg = 1.0 - vbd_jct / Q(PhiBD);
                if (MJD == 0.5)
                    sarg = 1.0 / sqrt(arg);
                else
                    sarg = exp(-MJD * log(arg));
                st0[B4S_QBD] = Q(PhiBD) * czbd * (1.0 - arg * sarg) / (1.0 - MJD);
                capbd = czbd * sarg;
            } else {
                st0[B4S_QBD] = 0.0;
                capbd = 0.0;
            }
            if (czbdsw > 0.0) {
                arg = 1.0 - vbd_jct / Q(PhiBSWD);
                if (MJSWD == 0.5)
                    sarg = 1.0 / sqrt(arg);
                else
                    sarg = exp(-MJSWD * log(arg));
                st0[B4S_QBD] += Q(PhiBSWD) * czbdsw * (1.0 - arg * sarg) / (1.0 - MJSWD);
                capbd += czbdsw * sarg;
            }
            if (czbdswg > 0.0) {
                arg = 1.0 - vbd_jct / Q(PhiBSWGD);
                if (MJSWGD == 0.5)
                    sarg = 1.0 / sqrt(arg);
                else
                    sarg = exp(-MJSWGD * log(arg));
                st0[B4S_QBD] += Q(PhiBSWGD) * czbdswg * (1.0 - arg * sarg) / (1.0 - MJSWGD);
                capbd += czbdswg * sarg;
            }
        } else {
            T0 = czbd + czbdsw + czbdswg;
            T1 = vbd_jct * (czbd * MJD / Q(PhiBD) + czbdsw * MJSWD / Q(PhiBSWD) +
                            czbdswg * MJSWGD / Q(PhiBSWGD));
            st0[B4S_QBD] = vbd_jct * (T0 + 0.5 * T1);
            capbd = T0 + T1;
        }
    }

    /* ---- convergence flag and state (b4ld.c:4060-4128) ---- */
    int noncon = 0;
    if ((!off) || (!(mode & NGSF_MODEINITFIX)))
        if (Check == 1)
            noncon = 1;
    st0[B4S_VDS] = vds;
    st0[B4S_VGS] = vgs;
    st0[B4S_VBS] = vbs;
    st0[B4S_VBD] = vbd;
    st0[B4S_VGES] = vges;
    st0[B4S_VGMS] = vgms;
    st0[B4S_VDBS] = vdbs;
    st0[B4S_VDBD] = vdbd;
    st0[B4S_VSBS] = vsbs;
    st0[B4S_VSES] = vses;
    st0[B4S_VDES] = vdes;
    st0[B4S_QDEF] = qdef;

    /* ---- companion models of the charges (b4ld.c:4129-4715) ---- */
    double ceqqg = 0, ceqqb = 0, ceqqd = 0;
    double gcggb = 0, gcgdb = 0, gcgsb = 0, gcgbb = 0, gcdgb = 0, gcddb = 0, gcdsb = 0, gcdbb = 0;
    double gcsgb = 0, gcsdb = 0, gcssb = 0, gcsbb = 0, gcbgb = 0, gcbdb = 0, gcbsb = 0, gcbbb = 0;
    if (ccn) {
        /* overlap capacitances, capMod 1/2 form (b4ld.c:4149-4174) */
        double cgdo, qgdo, cgso, qgso;
        {
            const double vgdx = vgd, vgsx = vgs;
            T0 = vgdx + B4_DELTA_1;
            T1 = sqrt(T0 * T0 + 4.0 * B4_DELTA_1);
            T2 = 0.5 * (T0 - T1);
            T3 = Q(weffCV) * Q(cgdl);
            T4 = sqrt(1.0 - 4.0 * T2 / Q(ckappad));
            cgdo = Q(cgdo) + T3 - T3 * (1.0 - 1.0 / T4) * (0.5 - 0.5 * T0 / T1);
            qgdo = (Q(cgdo) + T3) * vgdx - T3 * (T2 + 0.5 * Q(ckappad) * (T4 - 1.0));
            T0 = vgsx + B4_DELTA_1;
            T1 = sqrt(T0 * T0 + 4.0 * B4_DELTA_1);
            T2 = 0.5 * (T0 - T1);
            T3 = Q(weffCV) * Q(cgsl);
            T4 = sqrt(1.0 - 4.0 * T2 / Q(ckappas));
            cgso = Q(cgso) + T3 - T3 * (1.0 - 1.0 / T4) * (0.5 - 0.5 * T0 / T1);
            qgso = (Q(cgso) + T3) * vgsx - T3 * (T2 + 0.5 * Q(ckappas) * (T4 - 1.0));
        }
        if (nf != 1.0) {
            cgdo *= nf;
            cgso *= nf;
            qgdo *= nf;
            qgso *= nf;
        }
        const double ag0 = x.ag0;
        const double cgbo = Q(cgbo);
        double qsrc;
        if (bmode > 0) {
            qdrn -= qgdo;
            gcggb = (cggb + cgdo + cgso + cgbo) * ag0;
            gcgdb = (cgdb - cgdo) * ag0;
            gcgsb = (cgsb - cgso) * ag0;
            gcgbb = -(gcggb + gcgdb + gcgsb);
            gcdgb = (cdgb - cgdo) * ag0;
            gcsgb = -(cggb + cbgb + cdgb + cgso) * ag0;
            gcbgb = (cbgb - cgbo) * ag0;
            const double qgb = cgbo * vgb;
            qgate += qgdo + qgso + qgb;
            qbulk -= qgb;
            qsrc = -(qgate + qbulk + qdrn);
            gcddb = (cddb + capbd + cgdo) * ag0;
            gcdsb = cdsb * ag0;
            gcsdb = -(cgdb + cbdb + cddb) * ag0;
            gcssb = (capbs + cgso - (cgsb + cbsb + cdsb)) * ag0;
            gcdbb = -(gcdgb + gcddb + gcdsb);
            gcsbb = -(gcsgb + gcsdb + gcssb);
            gcbdb = (cbdb - capbd) * ag0;
            gcbsb = (cbsb - capbs) * ag0;
            gcbbb = -(gcbdb + gcbgb + gcbsb);
        } else {
            qsrc = qdrn - qgso;
            gcggb = (cggb + cgdo + cgso + cgbo) * ag0;
            gcgdb = (cgsb - cgdo) * ag0;
            gcgsb = (cgdb - cgso) * ag0;
            gcgbb = -(gcggb + gcgdb + gcgsb);
            gcdgb = -(cggb + cbgb + cdgb + cgdo) * ag0;
            gcsgb = (cdgb - cgso) * ag0;
            gcbgb = (cbgb - cgbo) * ag0;
            const double qgb = cgbo * vgb;
            qgate += qgdo + qgso + qgb;
            qbulk -= qgb;
            qdrn = -(qgate + qbulk + qsrc);
            gcddb = (capbd + cgdo - (cgsb + cbsb + cdsb)) * ag0;
            gcdsb = -(cgdb + cbdb + cddb) * ag0;
            gcsdb = cdsb * ag0;
            gcssb = (cddb + capbs + cgso) * ag0;
            gcdbb = -(gcdgb + gcddb + gcdsb);
            gcsbb = -(gcsgb + gcsdb + gcssb);
            gcbdb = (cbsb - capbd) * ag0;
            gcbsb = (cbdb - capbs) * ag0;
            gcbbb = -(gcbgb + gcbdb + gcbsb);
        }
        st0[B4S_QG] = qgate;
        st0[B4S_QD] = qdrn - st0[B4S_QBD];
        st0[B4S_QS] = qsrc - st0[B4S_QBS];
        st0[B4S_QB] = qbulk + st0[B4S_QBD] + st0[B4S_QBS];
        if (mode & NGSF_MODEINITTRAN) {
            st1[B4S_QB] = st0[B4S_QB];
            st1[B4S_QG] = st0[B4S_QG];
            st1[B4S_QD] = st0[B4S_QD];
        }
        dev_integrate(x, st0, st1, st2, B4S_QB);
        dev_integrate(x, st0, st1, st2, B4S_QG);
        dev_integrate(x, st0, st1, st2, B4S_QD);
        ceqqg = st0[B4S_CQG] - gcggb * vgb + gcgdb * vbd + gcgsb * vbs;
        ceqqd = st0[B4S_CQD] - gcdgb * vgb + gcddb * vbd + gcdsb * vbs;
        ceqqb = st0[B4S_CQB] - gcbgb * vgb + gcbdb * vbd + gcbsb * vbs;
        if (mode & NGSF_MODEINITTRAN) {
            st1[B4S_CQB] = st0[B4S_CQB];
            st1[B4S_CQG] = st0[B4S_CQG];
            st1[B4S_CQD] = st0[B4S_CQD];
        }
    }

    /* ---- equivalent currents and stamps (b4ld.c:4717-5232, 5435-5620) ---- */
    double Gmx, Gmbsx, FwdSum, RevSum, ceqdrn, ceqbd, ceqbs;
    double gbbdp, gbbsp, gbdpg, gbdpdp, gbdpb, gbdpsp, gbspg, gbspdp, gbspb, gbspsp;
    const double ggidls = -(Ggidld + Ggidlg + Ggidlb);
    const double ggisld = -(Ggisls + Ggislg + Ggislb);
    (void)ggidls; (void)ggisld;
    if (bmode >= 0) {
        Gmx = gm;
        Gmbsx = gmbs;
        FwdSum = Gmx + Gmbsx;
        RevSum = 0.0;
        ceqdrn = type * (cdrain - gds * vds - Gmx * vgs - Gmbsx * vbs);
        ceqbd = type * (csub + Igidl - (gbds + Ggidld) * vds - (gbgs + Ggidlg) * vgs -
                        (gbbs + Ggidlb) * vbs);
        ceqbs = type * (Igisl + Ggisls * vds - Ggislg * vgd - Ggislb * vbd);
        gbbdp = -(gbds);
        gbbsp = gbds + gbgs + gbbs;
        gbdpg = gbgs;
        gbdpdp = gbds;
        gbdpb = gbbs;
        gbdpsp = -(gbdpg + gbdpdp + gbdpb);
        gbspg = 0.0;
        gbspdp = 0.0;
        gbspb = 0.0;
        gbspsp = 0.0;
    } else {
        Gmx = -gm;
        Gmbsx = -gmbs;
        FwdSum = 0.0;
        RevSum = -(Gmx + Gmbsx);
        ceqdrn = -type * (cdrain + gds * vds + Gmx * vgd + Gmbsx * vbd);
        ceqbs = type * (csub + Igisl + (gbds + Ggisls) * vds - (gbgs + Ggislg) * vgd -
                        (gbbs + Ggislb) * vbd);
        ceqbd = type * (Igidl - Ggidld * vds - Ggidlg * vgs - Ggidlb * vbs);
        gbbsp = -(gbds);
        gbbdp = gbds + gbgs + gbbs;
        gbdpg = 0.0;
        gbdpsp = 0.0;
        gbdpb = 0.0;
        gbdpdp = 0.0;
        gbspg = gbgs;
        gbspsp = gbds;
        gbspb = gbbs;
        gbspdp = -(gbspg + gbspsp + gbspb);
    }
    double ceqjs, ceqjd;
    if (type > 0) {
        ceqjs = (cbs - gbs * vbs_jct);
        ceqjd = (cbd - gbd * vbd_jct);
    } else {
        ceqjs = -(cbs - gbs * vbs_jct);
        ceqjd = -(cbd - gbd * vbd_jct);
        ceqqg = -ceqqg;
        ceqqd = -ceqqd;
        ceqqb = -ceqqb;
    }
    const double mult_i = Q(mult_i), mult_q = Q(mult_q);
    const double gjbd = gbd, gjbs = gbs;
    const double gdpr = Q(drainConductance), gspr = Q(sourceConductance);
    if (Q(version47) == 0.0) {
        /* right-hand side: d', g', b', s' */
        sv[0 * svs] = (mult_i * (ceqjd - ceqbd - ceqdrn) - mult_q * ceqqd);
        sv[1 * svs] = -(mult_q * ceqqg);
        sv[2 * svs] = (mult_i * (ceqbd + ceqbs - ceqjd - ceqjs) - mult_q * ceqqb);
        sv[3 * svs] = (mult_i * (ceqdrn - ceqbs + ceqjs) + mult_q * (ceqqg + ceqqb + ceqqd));
        /* gate row (BSIM4_34..37) */
        sv[4 * svs] = mult_q * gcggb;
        sv[5 * svs] = mult_q * gcgdb;
        sv[6 * svs] = mult_q * gcgsb;
        sv[7 * svs] = mult_q * gcgbb;
        /* drain-prime row (BSIM4_44..50) */
        sv[8 * svs] = mult_i * (gdpr + gds + gbd + RevSum + gbdpdp) + mult_q * gcddb;
        sv[9 * svs] = -(mult_i * gdpr);
        sv[10 * svs] = mult_i * (Gmx + gbdpg) + mult_q * gcdgb;
        sv[11 * svs] = -(mult_i * (gds + FwdSum - gbdpsp) - mult_q * gcdsb);
        sv[12 * svs] = -(mult_i * (gjbd - Gmbsx - gbdpb) - mult_q * gcdbb);
        sv[13 * svs] = -(mult_i * gdpr);
        sv[14 * svs] = mult_i * gdpr;
        /* source-prime row (BSIM4_51..57) */
        sv[15 * svs] = -(mult_i * (gds + RevSum - gbspdp) - mult_q * gcsdb);
        sv[16 * svs] = mult_q * gcsgb + mult_i * (gbspg - Gmx);
        sv[17 * svs] = mult_i * (gspr + gds + gbs + FwdSum + gbspsp) + mult_q * gcssb;
        sv[18 * svs] = -(mult_i * gspr);
        sv[19 * svs] = -(mult_i * (gjbs + Gmbsx - gbspb) - mult_q * gcsbb);
        sv[20 * svs] = -(mult_i * gspr);
        sv[21 * svs] = mult_i * gspr;
        /* bulk-prime row (BSIM4_58..61) */
        sv[22 * svs] = mult_q * gcbdb - mult_i * (gjbd - gbbdp);
        sv[23 * svs] = mult_q * gcbgb - mult_i * gbgs;
        sv[24 * svs] = mult_q * gcbsb - mult_i * (gjbs - gbbsp);
        sv[25 * svs] = mult_i * (gjbd + gjbs - gbbs) + mult_q * gcbbb;
    } else {
        /* BSIM4v7 scales each stamp's whole sum by m and adds its terms in
         * the order of b4v7ld.c:4910-4925 and 5040-5084 (the terms of the
         * selectors this load rejects are zero and left out); a 4.7
         * instance has mult_i = mult_q = m */
        const double m = mult_i;
        sv[0 * svs] = m * (((ceqjd - ceqbd) - ceqdrn) - ceqqd);
        sv[1 * svs] = -(m * ceqqg);
        sv[2 * svs] = m * ((((ceqbd + ceqbs) - ceqjd) - ceqjs) - ceqqb);
        sv[3 * svs] = m * (((((ceqdrn - ceqbs) + ceqjs) + ceqqg) + ceqqb) + ceqqd);
        sv[4 * svs] = m * gcggb;
        sv[5 * svs] = m * gcgdb;
        sv[6 * svs] = m * gcgsb;
        sv[7 * svs] = m * gcgbb;
        sv[8 * svs] = m * (((((gdpr + gds) + gbd) + RevSum) + gcddb) + gbdpdp);
        sv[9 * svs] = -(m * gdpr);
        sv[10 * svs] = m * ((Gmx + gcdgb) + gbdpg);
        sv[11 * svs] = -(m * (((gds + FwdSum) - gcdsb) - gbdpsp));
        sv[12 * svs] = -(m * (((gjbd - Gmbsx) - gcdbb) - gbdpb));
        sv[13 * svs] = -(m * gdpr);
        sv[14 * svs] = m * gdpr;
        sv[15 * svs] = -(m * (((gds + RevSum) - gcsdb) - gbspdp));
        sv[16 * svs] = m * ((gcsgb - Gmx) + gbspg);
        sv[17 * svs] = m * (((((gspr + gds) + gbs) + FwdSum) + gcssb) + gbspsp);
        sv[18 * svs] = -(m * gspr);
        sv[19 * svs] = -(m * (((gjbs + Gmbsx) - gcsbb) - gbspb));
        sv[20 * svs] = -(m * gspr);
        sv[21 * svs] = m * gspr;
        sv[22 * svs] = m * ((gcbdb - gjbd) + gbbdp);
        sv[23 * svs] = m * (gcbgb - gbgs);
        sv[24 * svs] = m * ((gcbsb - gjbs) + gbbsp);
        sv[25 * svs] = m * (((gjbd + gjbs) + gcbbb) - gbbs);
    }
    /* GIDL (BSIM4_62..69) */
    sv[26 * svs] = mult_i * Ggidld;
    sv[27 * svs] = mult_i * Ggidlg;
    sv[28 * svs] = -(mult_i * (Ggidlg + Ggidld + Ggidlb));
    sv[29 * svs] = mult_i * Ggidlb;
    sv[30 * svs] = -(mult_i * Ggidld);
    sv[31 * svs] = -(mult_i * Ggidlg);
    sv[32 * svs] = mult_i * (Ggidlg + Ggidld + Ggidlb);
    sv[33 * svs] = -(mult_i * Ggidlb);
    /* GISL (BSIM4_70..77) */
    sv[34 * svs] = -(mult_i * (Ggisls + Ggislg + Ggislb));
    sv[35 * svs] = mult_i * Ggislg;
    sv[36 * svs] = mult_i * Ggisls;
    sv[37 * svs] = mult_i * Ggislb;
    sv[38 * svs] = mult_i * (Ggislg + Ggisls + Ggislb);
    sv[39 * svs] = -(mult_i * Ggislg);
    sv[40 * svs] = -(mult_i * Ggisls);
    sv[41 * svs] = -(mult_i * Ggislb);
#undef Q
    return noncon;
}
