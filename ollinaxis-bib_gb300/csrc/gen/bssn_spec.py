"""Pointwise algebra of the BSSN right-hand side in (rho, z), as symbolic
statements for the code generator (gen_rhs.py).

The formulas restate the reference's non-angmom BSSN branches:
  * covariant second derivatives of the lapse and its Laplacian,
    src/geometry/auxiliary_geometry.f90:1266-1324;
  * the Ricci tensor: conformal-factor part :1331-1469 and the conformal
    Ricci pieces of calc_conformalRicci1.f90:76-86, calc_conformalRicci2.f90:73-83,
    calc_conformalRicci3.f90:316-340, calc_conformalRicci4.f90:272-298;
    the Ricci scalar :1483-1493;
  * KT^ij, KT_i^m KT_mj and K_ij K^ij, :944-1031;
  * the divergence of the traceless curvature, calc_DIVKTA.f90:573-636;
  * the sources of trK, KTA/B/C and Delta_r/z without shift and matter
    terms, sources_geometry.f90:196-392,445-580 (the shift, matter,
    dissipation and boundary terms stay in rhs.cu);
  * the constraints of constraints.f90:55-149.

``algebra(x, let)`` receives the input symbols in ``x`` and a function
``let(name, expr)`` that turns an intermediate into a named temporary; the
generator optimises each temporary's polynomial (collection in r and 1/r,
multivariate Horner form, common subexpressions) and emits CUDA.
"""
import sympy as sp

INPUTS = [
    "r", "ir", "alpha", "chi", "Ac", "Bc", "Hc", "Cc", "trK", "kA", "kB", "kC", "kH",
    "Dlr", "Dlz", "gA", "gB", "gH", "gC", "lam", "Alam", "glam", "DDr", "DDz", "ipsi4", "eta",
    "da_r", "da_z", "da_rr", "da_zz", "da_rz", "dan_r", "dan_z",
    "dA_r", "dA_z", "dA_rr", "dA_zz", "dA_rz",
    "dB_r", "dB_z", "dB_rr", "dB_zz", "dB_rz",
    "dH_r", "dH_z", "dH_rr", "dH_zz", "dH_rz",
    "dC_r", "dC_z", "dC_rr", "dC_zz", "dC_rz",
    "Dr_phi", "Dz_phi", "Drr_phi", "Dzz_phi", "Drz_phi",
    "Dr_trK", "Dz_trK", "Dr_KTA", "Dz_KTA", "Dr_KTB", "Dz_KTB", "Dr_KTC", "Dz_KTC",
    "Dr_Dlr", "Dz_Dlr", "Dr_Dlz", "Dz_Dlz",
]

SOURCE_OUTPUTS = ["s_trK", "s_KTA", "s_KTB", "s_KTC", "s_Dlr", "s_Dlz"]
ANALYSIS_OUTPUTS = ["ham", "mom_r", "mom_z", "RSCAL", "KT2", "Lapla_alpha"]


def algebra(x, let):
    half, fourth, third = sp.Rational(1, 2), sp.Rational(1, 4), sp.Rational(1, 3)
    two, four, six = 2, 4, 6
    r, ir = x.r, x.ir
    r2, r3, r4, r5, ir2 = r ** 2, r ** 3, r ** 4, r ** 5, ir ** 2
    gA, gB, gH, gC = x.gA, x.gB, x.gH, x.gC
    Ac, Bc, Hc, Cc = x.Ac, x.Bc, x.Hc, x.Cc
    kA, kB, kC, kH = x.kA, x.kB, x.kC, x.kH
    Dlr, Dlz, lam, Alam, glam = x.Dlr, x.Dlz, x.lam, x.Alam, x.glam
    DDr, DDz, ipsi4, alpha, trK = x.DDr, x.DDz, x.ipsi4, x.alpha, x.trK
    Dr_phi, Dz_phi = x.Dr_phi, x.Dz_phi
    da_r, da_z = x.da_r, x.da_z
    dAr, dAz, dBr, dBz, dHr, dHz, dCr, dCz = x.dA_r, x.dA_z, x.dB_r, x.dB_z, x.dH_r, x.dH_z, x.dC_r, x.dC_z
    lamDef = let("lamDef", (Ac - Hc) * ir2)

    # lapse: covariant second derivatives (auxiliary_geometry.f90:1266-1309)
    aux1 = let("aux1", gA * da_r * Dr_phi + gB * da_z * Dz_phi + r * gC * (da_r * Dz_phi + da_z * Dr_phi))
    D2A = let("D2A", x.da_rr - da_r * gC * r2 * dCr
              - (da_z * gB * dCr + half * da_z * gC * dAr + da_r * gC * Cc - half * da_r * gC * dAz) * r
              - half * da_r * gA * dAr - da_z * gB * Cc + half * da_z * gB * dAz
              - two * (two * da_r * Dr_phi - Ac * aux1))
    D2B = let("D2B", x.da_zz - da_z * gC * r2 * dCz
              - (da_r * gA * dCz + half * da_r * gC * dBz - half * da_z * gC * dBr) * r
              + half * da_r * gA * dBr - half * da_z * gB * dBz
              - two * (two * da_z * Dz_phi - Bc * aux1))
    D2H = let("D2H", -(-half * da_r * gC * dHz - half * da_z * gC * dHr) * r
              + half * da_r * gA * dHr + da_z * gC * Hc + half * da_z * gB * dHz + da_r * gA * Hc * ir
              + two * Hc * aux1)
    D2C = let("D2C", x.da_rz * ir - half * da_r * gC * dBr - half * da_z * gC * dAz
              - (half * da_r * gA * dAz + half * da_z * gB * dBr) * ir
              - two * ((da_r * ir) * Dz_phi + da_z * (Dr_phi * ir) - Cc * aux1))
    Lapla = let("Lapla_alpha", (gA * D2A + gB * D2B + gH * D2H + two * r2 * gC * D2C) * ipsi4)

    # Ricci: second covariant derivatives of phi (times -2) (:1395-1420)
    RA0 = let("RA0", -two * (x.Drr_phi - Dr_phi * gC * r2 * dCr
              - (Dz_phi * gB * dCr + half * Dz_phi * gC * dAr + Dr_phi * gC * Cc - half * Dr_phi * gC * dAz) * r
              - half * Dr_phi * gA * dAr - Dz_phi * gB * Cc + half * Dz_phi * gB * dAz))
    RB0 = let("RB0", -two * (x.Dzz_phi - Dz_phi * gC * r2 * dCz
              - (Dr_phi * gA * dCz + half * Dr_phi * gC * dBz - half * Dz_phi * gC * dBr) * r
              + half * Dr_phi * gA * dBr - half * Dz_phi * gB * dBz))
    RH0 = let("RH0", -two * (-(-half * Dr_phi * gC * dHz - half * Dz_phi * gC * dHr) * r
              + half * Dr_phi * gA * dHr + Dz_phi * gC * Hc + half * Dz_phi * gB * dHz + Dr_phi * gA * Hc * ir))
    RC0 = let("RC0", -two * (x.Drz_phi * ir - half * Dr_phi * gC * dBr - half * Dz_phi * gC * dAz
              - (half * Dr_phi * gA * dAz + half * Dz_phi * gB * dBr) * ir))
    # trace (Laplacian of phi) and the contracted quadratic terms (:1424-1469)
    tr = let("trRphi", gA * RA0 + gB * RB0 + gH * RH0 + two * r2 * gC * RC0)
    q = let("qphi", -two * (gA * Dr_phi * Dr_phi + gB * Dz_phi * Dz_phi + two * r * gC * Dr_phi * Dz_phi))
    RA = RA0 + Ac * tr + four * (Dr_phi * Dr_phi) + two * Ac * q
    RB = RB0 + Bc * tr + four * (Dz_phi * Dz_phi) + two * Bc * q
    RH = RH0 + Hc * tr + two * Hc * q
    RC = RC0 + Cc * tr + four * (Dr_phi * Dz_phi) * ir + two * Cc * q
    # calc_conformalRicci1 (non-angmom)
    RA += -gC * x.dA_rz * r - half * gB * x.dA_zz - half * gA * x.dA_rr - half * gH * dAr * ir + gH * lamDef
    RB += -gC * x.dB_rz * r - half * gA * x.dB_rr - half * gB * x.dB_zz - half * gH * dBr * ir
    RH += -gC * x.dH_rz * r - half * gB * x.dH_zz - half * gA * x.dH_rr - half * gH * dHr * ir - gH * lamDef
    RC += -gC * x.dC_rz * r - half * gA * x.dC_rr - gC * dCz - half * gB * x.dC_zz + (-gA * dCr - half * gH * dCr) * ir
    # calc_conformalRicci2 (non-angmom)
    RA += Cc * x.Dr_Dlz * r + Ac * x.Dr_Dlr + half * (DDr * dAr + DDz * dAz)
    RB += Cc * x.Dz_Dlr * r + Bc * x.Dz_Dlz + half * (DDr * dBr + DDz * dBz)
    RH += half * (DDr * dHr + DDz * dHz) + Dlr * Hc * ir
    RC += half * Cc * (x.Dr_Dlr + x.Dz_Dlz) + half * (DDr * dCr + DDz * dCz) + half * (Cc * Dlr + Ac * x.Dz_Dlr + Bc * x.Dr_Dlz) * ir
    # calc_conformalRicci3 (non-angmom)
    RA += (2 * gB * gC * dCr * dCz + gC ** 2 * dAr * dCz + dAz * gC ** 2 * dCr) * r3 \
        + (2 * gB * gC * Cc * dCz - gB * gC * dCr * dBr + dAr * gC * gA * dCr + dAz * gC ** 2 * Cc) * r2 \
        + (dAz * gB * gC * dBr + dAz * gB * gA * dCr + dAr * gC * gA * Cc - gB * gC * Cc * dBr + dAz * gC * gA * dAr
           + gB ** 2 * dBr * dCz) * r \
        - half * gH ** 2 * dHr ** 2 - half * gB ** 2 * dBr ** 2 + gB * gA * Cc * dAz + half * dAr ** 2 * gA ** 2 \
        + (gH * dHr + gH ** 2 * Ac * dHr - 2 * gH ** 2 * dHr * Hc) * ir
    RB += (dBr * gC ** 2 * dCz + gC ** 2 * dBz * dCr + 2 * gA * gC * dCz * dCr) * r3 \
        + (2 * gA * gC * dCz * Cc - gA * gC * dCz * dAz + gC ** 2 * dBz * Cc + dBz * gC * gB * dCz) * r2 \
        + (dBr * gA * gC * dAz + gA ** 2 * dAz * dCr + dBr * gA * gB * dCz + dBr * gB * gC * dBz) * r \
        + half * gB ** 2 * dBz ** 2 + gA ** 2 * dAz * Cc - half * gA ** 2 * dAz ** 2 + gH ** 2 * dHz * Cc - half * gH ** 2 * dHz ** 2
    RH += -gC * dHz - r * glam * dHr
    RC += (gC ** 2 * dBr * dCr + gC * gB * dCz ** 2 + dAz * gC ** 2 * dCz + gC * gA * dCr ** 2) * r2 \
        + (-half * gC * gA * dCr * dAz + 2 * gC * gA * dCr * Cc - half * gC ** 2 * dBr * dAz - half * gC * gB * dCz * dBr
           + half * dBz * gB * gC * dCr + gC ** 2 * dBr * Cc + half * dBz * gC ** 2 * dAr + half * dAr * gA * gC * dCz) * r \
        + half * dBr * gC * gA * dAr + half * dBr * gB * gA * dCr + half * gB ** 2 * dBz * dCz + half * dAz * gA * gB * dCz \
        + half * gA ** 2 * dAr * dCr + half * dBr ** 2 * gB * gC + gC * gA * Cc ** 2 - half * gC * gA * Cc * dAz \
        + half * dAz * gB * gC * dBz + half * dAz ** 2 * gA * gC + half * dBz * gB * gC * Cc \
        + (half * gH ** 2 * Cc * dHr + half * gB * gA * dBr * Cc - half * gH ** 2 * dHz * dHr + half * gA ** 2 * dAr * Cc) * ir \
        + half * dHz * gH ** 2 * lam
    # calc_conformalRicci4 (non-angmom)
    RA += dAz * gC ** 2 * dCr * r3 \
        + (-half * dAz ** 2 * gC ** 2 + dAz * gC ** 2 * Cc + gB * gA * dCr ** 2 + half * dAr * gC ** 2 * dBr + dAr * gC * gA * dCr
           + gB * gC * dCr * dBr) * r2 \
        + (-dAz * gB * gA * dCr + 2 * gB * gA * dCr * Cc + gB * gC * Cc * dBr + dAr * gC * gA * Cc) * r \
        + fourth * gH ** 2 * dHr ** 2 - gB * gA * Cc * dAz + fourth * gB ** 2 * dBr ** 2 + gB * gA * Cc ** 2 \
        + fourth * dAr ** 2 * gA ** 2 + half * gB * gA * dAz ** 2
    RB += dBr * gC ** 2 * r3 * dCz \
        + (gA * gB * dCz ** 2 + half * dAz * gC ** 2 * dBz - half * gC ** 2 * dBr ** 2 + dBz * gC * gB * dCz + gA * gC * dCz * dAz) * r2 \
        - dBr * gA * gB * dCz * r + fourth * gA ** 2 * dAz ** 2 + half * gB * gA * dBr ** 2 + fourth * gH ** 2 * dHz ** 2 \
        + fourth * gB ** 2 * dBz ** 2
    RH += (-half * Cc * gC * gH * dHr + gH * gC * dHz * dHr) * r + half * gH * dHz ** 2 * gB \
        + 3 * half * gC * dHz + half * gH * gA * dHr ** 2 - half * Cc * gB * gH * dHz - half * gH * Ac * gC * dHz - Cc * gC \
        - half * gC * dHz + half * (2 * gA - gH - gH * Ac * gA) * dHr * ir + gH * lam * (1 - gA * Hc)
    RC += gC ** 2 * dCr * dCz * r3 \
        + (-half * dAz * gC ** 2 * dCz + gC ** 2 * Cc * dCz - half * gC ** 2 * dBr * dCr) * r2 \
        + (-half * gC ** 2 * dBr * Cc + fourth * dBz * gC ** 2 * dAr + half * dAr * gA * gC * dCz + half * gC * gB * dCz * dBr
           + 3 * fourth * gC ** 2 * dBr * dAz + half * dBz * gB * gC * dCr + half * gC * gA * dCr * dAz) * r \
        + half * dAz * gA * gB * dCz + half * dBz * gB * gC * Cc + half * gC * gA * Cc * dAz + half * dBr * gB * gA * dCr \
        + (fourth * gH ** 2 * dHz * dHr + half * gB * gA * dBr * Cc + fourth * gA ** 2 * dAr * dAz + fourth * dBz * gB ** 2 * dBr
           - half * gB * gA * dAz * dBr) * ir
    RA = let("RA", RA)
    RB = let("RB", RB)
    RH = let("RH", RH)
    RC = let("RC", RC)
    RSCAL = let("RSCAL", (gA * RA + gB * RB + gH * RH + two * r2 * gC * RC) * ipsi4)

    # traceless curvature contractions (:944-1031)
    KT_up_rr = let("KT_up_rr", (2 * gA * gC * kC + gC ** 2 * kB) * r2 + gA ** 2 * kA)
    KT_up_zz = let("KT_up_zz", (gC ** 2 * kA + 2 * gC * gB * kC) * r2 + gB ** 2 * kB)
    KT_up_rz = let("KT_up_rz", gC ** 2 * r3 * kC + (gC * gA * kA + gB * gA * kC + gB * gC * kB) * r)
    KT2_A = let("KT2_A", (2 * kA * gC * kC + kC ** 2 * gB) * r2 + gA * kA ** 2)
    KT2_B = let("KT2_B", (kC ** 2 * gA + 2 * kC * gC * kB) * r2 + gB * kB ** 2)
    KT2_C = let("KT2_C", kC ** 2 * gC * r2 + kA * gA * kC + kA * gC * kB + kC * gB * kB)
    KT2 = let("KT2", gA * KT2_A + gB * KT2_B + gH * kH ** 2 * gH + two * gC * KT2_C * r2)
    K2 = KT2 + third * trK ** 2

    # divergence of KT (calc_DIVKTA.f90, non-angmom)
    dkAr, dkAz, dkBr, dkBz, dkCr, dkCz = x.Dr_KTA, x.Dz_KTA, x.Dr_KTB, x.Dz_KTB, x.Dr_KTC, x.Dz_KTC
    DIV_KT_r = -gC ** 3 * dCz * kC * r5 - gA * gC ** 2 * kC * dCr * r4 \
        + (gC ** 2 * dkCz - half * gC ** 3 * dBz * kA - gA * gC ** 2 * kC * Cc - half * gC ** 3 * dAz * kB - gA * dCz * gC ** 2 * kA
           - gA * dCz * gC * gB * kC - gC ** 2 * dCz * gB * kB - gC ** 2 * dBz * gB * kC - gA * dAz * gC ** 2 * kC) * r3 \
        + (2 * gA * gC * dkCr - Dlr * gC * kC - gC * dBr * gB * gA * kC - gB * gA ** 2 * kC * dCr - dAr * gA ** 2 * gC * kC
           - gC * gA ** 2 * kA * dCr + gC ** 2 * dkBr - gA * gB * gC * kB * dCr - half * gA * dAr * gC ** 2 * kB
           - half * gC ** 2 * dBr * gA * kA) * r2 \
        + (2 * gA * gC * kC + gA * gC * dkAz - gC * gA ** 2 * kA * Cc + gC * gH * kC - half * gH ** 2 * kH * gC * dHz
           - Dlz * gC * kB - gB * gA ** 2 * kC * Cc - half * gA ** 2 * dAz * gC * kA + gC * gB * dkBz + gA * gB * dkCz
           - Dlz * gA * kC - gA * gB * gC * kB * Cc - gC * gH ** 2 * kH * Cc - half * gC * dBz * gB ** 2 * kB) * r \
        - half * gA * dBr * gB ** 2 * kB - half * gH ** 2 * kH * gA * dHr - Dlr * gA * kA + gA ** 2 * dkAr \
        - half * gA ** 3 * dAr * kA + r * gH * (gA * Alam + gH * kH * Cc * gC)
    DIV_KT_z = -r5 * gC ** 3 * kC * dCr + (-gC ** 3 * kC * Cc - dCz * gC ** 2 * gB * kC) * r4 \
        + (gC ** 2 * dkCr - gB * gC ** 2 * kB * dCr - gC * gB * gA * kC * dCr - half * gC ** 3 * dBr * kA - gC ** 2 * gA * kA * dCr
           - half * dAr * gC ** 3 * kB - dAr * gA * gC ** 2 * kC - gB * dBr * gC ** 2 * kC) * r3 \
        + (-gB * dCz * gC * gA * kA + gC ** 2 * kC - dBz * gC * gB ** 2 * kC - Dlz * gC * kC - gC * dCz * gB ** 2 * kB
           + gC ** 2 * dkAz + 2 * gC * gB * dkCz - gC ** 2 * gA * kA * Cc - dCz * gB ** 2 * gA * kC - half * dAz * gB * gC ** 2 * kB
           - gC * dAz * gB * gA * kC - gB * gC ** 2 * kB * Cc - half * gB * dBz * gC ** 2 * kA - gC * gB * gA * kC * Cc) * r2 \
        + (gB * gC * dkBr + gB * gA * dkCr + gC * gA * dkAr - half * gH ** 2 * kH * gC * dHr - Dlr * gB * kC - Dlr * gC * kA
           - half * gB ** 2 * dBr * gC * kB - half * gC * dAr * gA ** 2 * kA) * r \
        + gC * gH * kA + gB * gA * kC - half * dBz * gB ** 3 * kB + gB ** 2 * dkBz - Dlz * gB * kB - gC * gH ** 2 * kH * Ac \
        - half * gB * dAz * gA ** 2 * kA - half * gH ** 2 * kH * gB * dHz - gC * gH * kH + gB * gH * kC - gB * gH ** 2 * kH * Cc
    DIVA_KT_r = -r5 * gC ** 3 * dCz * kC + (-gC ** 3 * dCr * kB - gC ** 3 * dBr * kC - 3 * gC ** 2 * dCr * gA * kC) * r4 \
        + (-gC ** 3 * Cc * kB - 2 * gA * dCz * gC ** 2 * kA - 3 * gC ** 2 * Cc * gA * kC + gC ** 2 * dkCz - gC ** 2 * dAz * gA * kC
           - 3 * gA * dCz * gC * gB * kC - 2 * gC ** 2 * dBz * gB * kC - gC ** 3 * dBz * kA - gC ** 2 * dCz * gB * kB) * r3 \
        + (-gA * dBr * gC ** 2 * kA - gA * gB * gC * kB * dCr + 2 * gA * gC * dkCr - 2 * gC * dCr * gA ** 2 * kA - Dlr * gC * kC
           + gC ** 2 * dkBr - gC ** 2 * dBr * gB * kB - 2 * gA ** 2 * dAr * gC * kC - gA * dAr * gC ** 2 * kB
           - gB * gA ** 2 * kC * dCr - gA * dBr * gC * gB * kC) * r2 \
        + (-gA * dCz * gB ** 2 * kB - gB * gA ** 2 * kC * Cc - gC * dBz * gB ** 2 * kB + 2 * gA * gC * kC + gC * gB * dkBz
           + gC * gH * kC + gA * gC * dkAz + gA * gB * dkCz - gA * dAz * gB * gC * kB - gC * gH ** 2 * kH * Cc - Dlz * gC * kB
           - gA ** 2 * dAz * gB * kC - 2 * gC * Cc * gA ** 2 * kA - Dlz * gA * kC - gA ** 2 * dAz * gC * kA - gA * gB * gC * kB * Cc) * r \
        - dAr * gA ** 3 * kA - Dlr * gA * kA + gA ** 2 * dkAr + r * gA * gH * (Alam - lam * gH * kH)
    DIVA_KT_z = -r5 * gC ** 3 * kC * dCr \
        + (-3 * dCz * gC ** 2 * gB * kC - dAz * gC ** 3 * kC - dCz * gC ** 3 * kA - gC ** 3 * kC * Cc) * r4 \
        + (-3 * gC * gB * gA * kC * dCr - 2 * dAr * gA * gC ** 2 * kC + gC ** 2 * dkCr - gB * dBr * gC ** 2 * kC
           - dAr * gC ** 3 * kB - 2 * gB * gC ** 2 * kB * dCr - gC ** 2 * gA * kA * dCr) * r3 \
        + (-gC * dAz * gB * gA * kC - gC ** 2 * gA * kA * Cc - 2 * dBz * gC * gB ** 2 * kC - dAz * gC ** 2 * gA * kA
           - dAz * gB * gC ** 2 * kB - 3 * gC * gB * gA * kC * Cc - 2 * gC * dCz * gB ** 2 * kB - Dlz * gC * kC
           - dCz * gB ** 2 * gA * kC + gC ** 2 * kC + gC ** 2 * dkAz + 2 * gC * gB * dkCz - gB * dCz * gC * gA * kA
           - gB * dBz * gC ** 2 * kA - 2 * gB * gC ** 2 * kB * Cc) * r2 \
        + (-Dlr * gB * kC + gB * gA * dkCr + gC * gA * dkAr + gB * gC * dkBr - gB ** 2 * dBr * gC * kB - Dlr * gC * kA
           - gB ** 2 * dBr * gA * kC - gC * dAr * gA ** 2 * kA - gB * dBr * gC * gA * kA - gB * gA ** 2 * kA * dCr) * r \
        - Dlz * gB * kB - gB * gH ** 2 * kH * Cc + gB ** 2 * dkBz - gC * gH ** 2 * kH * Ac - gB * gA ** 2 * kA * Cc + gB * gH * kC \
        + gC * gH * kA + gB * gA * kC - dBz * gB ** 3 * kB
    DIV_KT_r = let("DIV_KT_r", DIV_KT_r)
    DIV_KT_z = let("DIV_KT_z", DIV_KT_z)
    DIVA_KT_r = let("DIVA_KT_r", DIVA_KT_r)
    DIVA_KT_z = let("DIVA_KT_z", DIVA_KT_z)

    # sources without shift and matter terms (sources_geometry.f90)
    trterm = let("trterm", -Lapla + alpha * RSCAL)
    out = {}
    out["s_trK"] = -Lapla + alpha * K2
    out["s_KTA"] = alpha * (trK * kA - two * KT2_A) + (-D2A + alpha * RA) * ipsi4 - third * Ac * trterm
    out["s_KTB"] = alpha * (trK * kB - two * KT2_B) + (-D2B + alpha * RB) * ipsi4 - third * Bc * trterm
    out["s_KTC"] = alpha * (trK * kC - two * KT2_C) + (-D2C + alpha * RC) * ipsi4 - third * Cc * trterm
    # the lapse gradient of the Delta sources is the one maximalslicing.f90
    # recomputes (dan_*); D2cov_alpha and Lapla_alpha above keep the values of
    # the last ``auxiliary`` call (da_*); the two differ only in the first
    # stage after a maximal-slicing solve
    out["s_Dlr"] = -two * (KT_up_rr * x.dan_r + KT_up_rz * x.dan_z) - two * alpha * DIVA_KT_r \
        + x.eta * alpha * (DIV_KT_r + six * (KT_up_rr * Dr_phi + KT_up_rz * Dz_phi) - two * third * (gA * x.Dr_trK + r * gC * x.Dz_trK))
    out["s_Dlz"] = -two * (KT_up_rz * x.dan_r + KT_up_zz * x.dan_z) - two * alpha * DIVA_KT_z \
        + x.eta * alpha * (DIV_KT_z + six * (KT_up_rz * Dr_phi + KT_up_zz * Dz_phi) - two * third * (r * gC * x.Dr_trK + gB * x.Dz_trK))
    # constraints (constraints.f90:55-149), vacuum part
    out["ham"] = RSCAL - KT2 + two * third * trK ** 2
    out["mom_r"] = DIV_KT_r + six * (KT_up_rr * Dr_phi + KT_up_rz * Dz_phi) - two * third * (gA * x.Dr_trK + r * gC * x.Dz_trK)
    out["mom_z"] = DIV_KT_z + six * (KT_up_rz * Dr_phi + KT_up_zz * Dz_phi) - two * third * (r * gC * x.Dr_trK + gB * x.Dz_trK)
    out["RSCAL"] = RSCAL
    out["KT2"] = KT2
    out["Lapla_alpha"] = Lapla
    return out
