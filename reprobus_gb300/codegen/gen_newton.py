"""Generates csrc/newton_gen.cuh: residual, analytic Jacobian and sparse LU of
the REPROBUS chemistry step equations, for the per-cell Newton solver.

The equations are the fixed point of one pass of the reference's iteration
(src/reprobus_l137_20230723.f:1350-2372): the unknowns are the 42 updated
transported slots ck(1..42) and the 15 short-lived slots cc(1..15),
x = (ck, cc). The reference evaluates each short-lived formula with values
already updated earlier in the same pass (Gauss-Seidel order, three species
damped by 1/2); at a fixed point every value equals its update, so the same
fixed point solves the "Jacobi form" written here, in which every formula
reads the current iterate x:

  short-lived s:  R_s = x_s - g_s(x)        (g_s: the reference's formula for
                                              cc(s), undamped)
  transported n:  R_n = x_n (1 + dt pe_n(x)) - ck0_n - dt pr_n(x)
                  (families, whose loss the reference divides by ck_n:
                   R_n = x_n + dt L_n(x) - ck0_n - dt pr_n(x))

so the Jacobian is sparse (an entry (i,j) exists when x_j appears in the
formula of unknown i). Day (sza <= 95) and night cells have separate
equations (the branch at :1352).

The generator differentiates the formulas symbolically (sympy, chain rule
over the named intermediates), takes the union sparsity pattern of day and
night, orders the unknowns by minimum degree, computes the LU fill pattern
(no pivoting), and emits straight-line code:

  nt_residual_day/night(F, x, R)    FP64
  nt_jacobian_day/night<T>(F, x, J) T = double or float, J in the LU slots
  nt_lu<T>(J), nt_solve<T>(J, b)

Run: python -m reprobus_gb300.codegen.gen_newton   (writes csrc/newton_gen.cuh)
"""
from __future__ import annotations

import os
import sys

import sympy as sp
from sympy.printing.c import C99CodePrinter

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from reprobus_gb300.species import LONG, PHOT, RATES, SHORT  # noqa: E402

NL, NS = 42, 15
NX = NL + NS
X = [sp.Symbol(f"x[{j}]") for j in range(NX)]
XIDX = {s: j for j, s in enumerate(X)}


def CK(m):
    return X[m - 1]


def CC(s):
    return X[NL + s - 1]


KS = {n: sp.Symbol(f"K[K_{n}]") for n in RATES}
TJS = {n: sp.Symbol(f"tj[J_{n}]") for n in PHOT}
HETS = [sp.Symbol(f"het[{i}]") for i in range(9)]
CK0 = [sp.Symbol(f"ck0[{m}]") for m in range(NL)]
F = {n: sp.Symbol(f"F.{n}") for n in ("o2", "n2", "h2", "co2", "hnm", "parthno3", "parth2o", "parthcl",
                                       "parthbr", "rain_hno3", "rain_hcl", "rain_hbr", "rain_h2o2", "dt")}


def K(n):
    return KS[n]


def TJ(n):
    return TJS[n]


def HET(m):
    return HETS[m - 1]


class Model:
    """SSA list of named intermediates with their sparse gradients."""

    def __init__(self, tag):
        self.tag = tag
        self.stmts = []   # (kind, sym, payload, grad)
        self.grad = {}
        self.n = 0

    def dsym(self, u, j):
        return sp.Symbol(f"d_{u.name}_{j}")

    def gradient(self, expr):
        out = {}
        for u in expr.free_symbols:
            if u in XIDX:
                d = sp.diff(expr, u)
                if d != 0:
                    out[XIDX[u]] = out.get(XIDX[u], 0) + d
            elif u in self.grad:
                du = sp.diff(expr, u)
                if du == 0:
                    continue
                for j in self.grad[u]:
                    out[j] = out.get(j, 0) + du * self.dsym(u, j)
        return {j: g for j, g in out.items() if g != 0}

    def let(self, name, expr):
        expr = sp.sympify(expr)
        s = sp.Symbol(f"{self.tag}_{name}")
        g = self.gradient(expr)
        self.stmts.append(("let", s, expr, g))
        self.grad[s] = g
        return s

    def let_min(self, name, a, b, op="min"):
        a, b = sp.sympify(a), sp.sympify(b)
        s = sp.Symbol(f"{self.tag}_{name}")
        ga, gb = self.gradient(a), self.gradient(b)
        keys = set(ga) | set(gb)
        g = {j: (ga.get(j, sp.Integer(0)), gb.get(j, sp.Integer(0))) for j in keys}
        self.stmts.append((op, s, (a, b), g))
        self.grad[s] = {j: None for j in keys}
        return s

    def let_max(self, name, a, b):
        return self.let_min(name, a, b, op="max")

    def let_sel(self, name, lhs, rhs, a, b):
        """value = (lhs > rhs) ? a : b, derivative of the selected branch."""
        lhs, rhs, a, b = (sp.sympify(v) for v in (lhs, rhs, a, b))
        s = sp.Symbol(f"{self.tag}_{name}")
        ga, gb = self.gradient(a), self.gradient(b)
        keys = set(ga) | set(gb)
        g = {j: (ga.get(j, sp.Integer(0)), gb.get(j, sp.Integer(0))) for j in keys}
        self.stmts.append(("sel", s, (lhs, rhs, a, b), g))
        self.grad[s] = {j: None for j in keys}
        return s


def build(day: bool):
    """The Jacobi-form equations of one pass; returns (model, residual list)."""
    m = Model("D" if day else "N")
    o2, n2, h2, hnm, co2, dt = F["o2"], F["n2"], F["h2"], F["hnm"], F["co2"], F["dt"]
    parthno3, parth2o, parthcl, parthbr = F["parthno3"], F["parth2o"], F["parthcl"], F["parthbr"]
    rain_hno3, rain_hcl, rain_hbr, rain_h2o2 = F["rain_hno3"], F["rain_hcl"], F["rain_hbr"], F["rain_h2o2"]
    rain_hno4 = rain_ch2o = rain_ch3o2h = 0
    a3et, a23a, a23b, a23c = sp.Float(1.2e-10), sp.Float(7.2e-11), sp.Float(6.9e-12), sp.Float(1.6e-12)
    a23 = sp.Float(7.2e-11 + 6.9e-12 + 1.6e-12)
    g = {}   # short-lived formulas g_s (index s 1..15)
    if day:
        g[15] = ((K("c2") * CC(2) + K("c1a") * CC(1) + K("d5") * CC(3)) * CK(2)) / (K("c4") * o2 + K("c3") * CC(4))
        ch3o = m.let("ch3o", (K("c1b") * CC(1) * CK(2) + (K("c5") * CC(8) + 2 * K("c14") * CK(29) + K("c18") * CC(11))
                              * CK(29) + TJ("ch3o2h") * CK(30)) / (K("c15") * o2))
        hco = m.let("hco", (K("c8") * CC(2) + K("c9") * CC(4) + K("c10") * CC(3) + K("c19") * CC(9) + TJ("ch2o_hco"))
                    * CK(28) / (K("c12") * o2))
        r1 = m.let("r1", (TJ("o3_o1d") + TJ("o3_o3p") + K("a2") * CC(14) + K("a6") * CC(2) + K("a6b") * CC(6)
                          + K("b4") * CC(8) + K("d2") * CC(3)) / (K("hk2") * o2))
        g[5] = CK(8) / (1 + r1)
        g[4] = r1 * CC(5)
        r3 = TJ("o3_o1d") / (K("hk4") * n2 + K("hk5") * o2)
        g[1] = r3 * CC(5)
        r4 = m.let("r4", (K("a5") * CC(4) + K("a36") * CK(9) + K("a19") * h2)
                   / (K("a1") * o2 + K("a2") * CC(5) + a23 * CC(6)))
        g[14] = r4 * CC(2)
        r7 = m.let("r7", TJ("no") / (K("b7") * o2 + K("b6") * CC(8)))
        r8 = m.let("r8", (K("b9") * CC(5)) / (TJ("no3_no") + TJ("no3_no2") + K("b12") * CC(7)))
        r5 = m.let("r5", (TJ("no2") + K("b3") * CC(4) + TJ("no3_no") * r8)
                   / (K("b4") * CC(5) + K("a26") * CC(6) + K("d4") * CC(11) + K("e4") * CC(12) + K("c5") * CK(29)))
        g[7] = CK(21) / (1 + r5 + r7 * r5 + r8)
        g[8] = r5 * CC(7)
        g[10] = r7 * CC(8)
        g[13] = r8 * CC(7)
        r6 = m.let("r6", (K("a6") * CC(5) + K("a30") * CK(17) + K("c8") * CK(28) + K("d8") * CC(11)
                          + K("e10") * CC(12) + K("a1") * o2 * r4)
                   / (a23 * CC(14) + K("a6b") * CC(5) + K("a7") * CC(4) + K("a26") * CC(8) + 2 * K("a27") * CC(6)
                      + K("a17") * CC(2) + K("d7") * CC(3) + K("d10") * CC(3) + K("d33") * CC(11) + K("e7") * CC(9)
                      + K("e15") * CC(12)))
        g[6] = CC(2) * r6
        r13 = m.let("r13", K("d31") * CC(7) / (TJ("clono2_cl") + TJ("clono2_clo") + K("d32") * CC(4)
                                               + HET(1) * CK(3) + HET(2) * CK(13)))
        r9 = m.let("r9", (K("d33") * CC(6) + HET(1) * CK(3) * r13) / (HET(5) * CK(13) + K("d35") * CC(4)
                                                                        + TJ("hocl")))
        r10 = m.let("r10", (K("d60") * CC(11)) / (K("d61") * hnm + TJ("cl2o2")))
        r12 = m.let("r12", K("e5c") * CC(12) / TJ("brcl"))
        r11 = m.let("r11", (K("d3") * CC(4) + K("d4") * CC(8) + K("d8") * CC(2) + K("c18") * CK(29)
                            + K("e5b") * CC(12) + TJ("clono2_cl") * r13 + TJ("hocl") * r9 + 2 * TJ("cl2o2") * r10
                            + TJ("brcl") * r12)
                    / (K("d2") * CC(5) + K("d5") * CK(2) + K("d7") * CC(6) + K("d10") * CC(6) + K("d37") * CK(15)))
        g[11] = CK(23) / (1 + r11)
        g[3] = r11 * CC(11)
        r27 = m.let("r27", K("e13") * CC(7) / (TJ("brono2") + K("e8") * CC(4)))
        r28 = m.let("r28", K("e15") * CC(6) / (TJ("hobr") + K("e16") * CC(4)))
        r29 = m.let("r29", K("e5c") * CC(11) / TJ("brcl"))
        r30 = m.let("r30", (K("e3") * CC(4) + K("e4") * CC(8) + K("e5a") * CC(11) + K("e5b") * CC(11)
                            + 2 * K("e6") * CC(12) + K("e10") * CC(2) + TJ("bro") + TJ("brono2") * sp.Float(0.85) * r27
                            + TJ("hobr") * r28 + TJ("brcl") * r29)
                    / (K("e2") * CC(5) + K("e7") * CC(6) + K("c19") * CK(28)))
        g[12] = CK(24) / (1 + r30)
        g[9] = r30 * CC(12)
        coea = m.let("coea", 2 * K("a31") + 2 * (K("a17") + K("a27") * r6 + (a23b + a23c) * r4) * r6)
        coeb = m.let("coeb", K("b27") * CK(5) * parthno3 + K("b22") * CC(7) + K("b28") * CK(22)
                     + K("b23") * CC(7) * r6 + K("c2") * CK(2) + K("c7") * CK(29) * r6 + K("c8") * CK(28)
                     + K("c17a") * CK(30) + K("d7") * CC(3) * r6 + K("d9") * CC(11) + K("d11") * CK(13) * parthcl
                     + K("d33") * CC(11) * r6 + K("d34") * CK(15) + K("e11") * CK(19) * parthbr
                     + K("e7") * CC(9) * r6 + K("e15") * CC(12) * r6)
        coec = m.let("coec", 2 * (K("a1et") * CC(1) + TJ("h2o")) * CK(3) * parth2o
                     + ((K("c1a") + K("c1b")) * CK(2) + 2 * a3et * h2) * CC(1)
                     + K("c3") * CC(15) * CC(4) + TJ("ch3o2h") * CK(30) + K("c15") * ch3o * o2
                     + (TJ("ch2o_hco") + K("c9") * CC(4)) * CK(28) + K("c12") * hco * o2
                     + TJ("hno3") * CK(5) * parthno3 + (K("b24") * hnm + TJ("hno4")) * CK(22)
                     + (K("d35") * CC(4) + K("d37") * CC(3) + TJ("hocl")) * CK(15)
                     + 2 * TJ("h2o2") * CK(17) + K("d6") * h2 * CC(3) + TJ("hobr") * CK(26)
                     + K("e16") * CC(4) * CK(26) + TJ("hbr") * CK(19))
        argum = m.let_max("argum", coeb * coeb + 4 * coea * coec, 0)
        g[2] = (sp.sqrt(argum) - coeb) / (2 * coea)
        day_f = 1
    else:
        for s in (14, 15, 1, 4, 2, 3, 6, 8, 10, 9):
            g[s] = sp.Integer(0)
        ch3o = hco = sp.Integer(0)
        g[5] = CK(8)
        # F:1721-1730: NO2 <- NOx/(1 + r8), r8 = b9 O3/(b12 max(NO2, 1e-30)),
        # NO3 = r8 * (updated NO2). The fixed point of this 1-D map is unique:
        # NO2 = NOx - c (c = b9 O3/b12) when that exceeds 1e-30, else inside the
        # clamp NO2 = NOx/(1 + c/1e-30), NO3 = NOx (c/1e-30)/(1 + c/1e-30)
        # (written as NOx 1e-30/(1e-30 + c) so that no intermediate overflows FP32)
        cno = m.let("cno", K("b9") * CC(5) / K("b12"))
        dno = m.let("dno", CK(21) - cno)
        eps = sp.Float(1e-30)
        g[7] = m.let_sel("no2", dno, eps, dno, CK(21) * eps / (eps + cno))
        g[13] = m.let_sel("no3", dno, eps, cno, CK(21) * cno / (eps + cno))
        g[11] = m.let_max("clo", CK(23), 0)
        g[12] = m.let_max("bro", CK(24), 0)
        day_f = 0

    # production / loss, F:1758-2358 (family losses L before the division by ck)
    pr, pe, fam = {}, {}, {}
    pr[1] = 0
    pe[1] = TJ("n2o") + (K("b38") + K("b39")) * CC(1)
    pr[2] = 0
    pe[2] = K("c2") * CC(2) + K("c1a") * CC(1) + K("c1b") * CC(1) + K("c1c") * CC(1) + K("d5") * CC(3)
    pr[3] = (K("c2") * CC(2) * CK(2) + K("c8") * CC(2) * CK(28) + K("c17a") * CK(30) * CC(2)
             + K("c17b") * CK(30) * CC(2) + (K("a17") * CC(2) + a23c * CC(14)) * CC(6) + K("a19") * CC(2) * h2
             + K("a30") * CC(2) * CK(17) + K("a31") * CC(2) * CC(2) + K("b27") * CC(2) * CK(5) * parthno3
             + K("d11") * CC(2) * CK(13) * parthcl)
    pe[3] = (TJ("h2o") + K("a1et") * CC(1)) * parth2o
    pr[4] = 2 * K("b39") * CC(1) * CK(1)
    fam[4] = 2 * K("b6") * CC(10) * CC(8) + rain_hno3 * CK(5) + rain_hno4 * CK(22)
    pr[5] = (K("b22") * CC(2) * CC(7) + HET(1) * CK(14) * CK(3) + HET(2) * CK(14) * CK(13)
             + 2 * HET(3) * CK(6) * CK(3) + HET(4) * CK(6) * CK(13) + HET(6) * CK(20) * CK(3))
    pe[5] = (TJ("hno3") + K("b27") * CC(2)) * parthno3 + rain_hno3
    pr[6] = K("b12") * CC(13) * CC(7)
    pe[6] = TJ("n2o5") + K("b32") * hnm + HET(3) * CK(3) + HET(4) * CK(13)
    pr[7] = (3 * (TJ("cfc11") + K("d90") * CC(1)) * CK(31) + 2 * (TJ("cfc12") + K("d91") * CC(1)) * CK(32)
             + 3 * (TJ("cfc113") + K("d92") * CC(1)) * CK(33) + 4 * (TJ("ccl4") + K("d93") * CC(1)) * CK(34)
             + 3 * (TJ("ch3ccl3") + K("d94") * CC(2)) * CK(35) + (TJ("ch3cl") + K("d95") * CC(2)) * CK(36)
             + (TJ("hcfc22") + K("d96") * CC(1) + K("d97") * CC(2)) * CK(37)
             + (TJ("h1211") + K("e52") * CC(1)) * CK(39))
    fam[7] = rain_hcl * CK(13)
    ratio = TJ("cl2o2") / (TJ("cl2o2") + K("d61") * hnm)
    pr[8] = 2 * TJ("o2") * o2 + K("a26") * CC(6) * CC(8) + K("c5") * CC(8) * CK(29)
    t06 = m.let_min("t06", TJ("hocl") * CK(15), K("d33") * CC(6) * CC(11))
    t07 = m.let_min("t07", K("e5c") * CC(12) * CC(11), TJ("brcl") * CK(27))
    t09 = m.let_min("t09", K("e15") * CC(12) * CC(6), TJ("hobr") * CK(26))
    jno3 = TJ("no3_no") / sp.Max(TJ("no3_no") + TJ("no3_no2"), sp.Float(1e-30))
    fam[8] = (2 * K("hk1") * CC(4) * CC(4) + 2 * K("hk3") * CC(5) * CC(4) + 2 * K("b3") * CC(7) * CC(4)
              + 2 * K("d3") * CC(11) * CC(4) + 2 * K("d60") * ratio * CC(11) * CC(11) + t06 + 2 * t07
              + 2 * K("e5b") * CC(12) * CC(11) * day_f + t09 + 2 * K("e6") * CC(12) * CC(12) * day_f
              + 2 * jno3 * TJ("clono2_cl") * CK(14)
              + (K("a2") * CC(14) + K("a6") * CC(2) + K("a6b") * CC(6)) * CC(5)
              + (K("a5") * CC(2) + K("a7") * CC(6)) * CC(4)
              + 2 * K("b9") * CC(7) * CC(5) * jno3)
    pr[9] = TJ("co2") * co2 + TJ("ch2o_co") * CK(28) + K("c12") * hco * o2
    pe[9] = K("a36") * CC(2)
    pr[10] = K("e5a") * CC(12) * CC(11)
    pe[10] = TJ("oclo")
    pr[11] = pe[11] = pr[12] = pe[12] = 0
    pr[13] = (K("c10") * CK(28) + K("d5") * CK(2) + K("d7") * CC(6) + K("d6") * h2) * CC(3) + K("d9") * CC(2) * CC(11)
    pe[13] = ((TJ("hcl") + K("d11") * CC(2)) * parthcl + HET(2) * CK(14) + HET(4) * CK(6) + HET(5) * CK(15)
              + HET(7) * CK(26) + rain_hcl)
    pr[14] = K("d31") * CC(7) * CC(11)
    pe[14] = TJ("clono2_cl") + TJ("clono2_clo") + K("d32") * CC(4) + HET(1) * CK(3) + HET(2) * CK(13)
    pr[15] = K("d33") * CC(6) * CC(11) + HET(1) * CK(14) * CK(3)
    pe[15] = (TJ("hocl") + K("d34") * CC(2) + K("d35") * CC(4) + K("d37") * CC(3) + HET(5) * CK(13)
              + HET(9) * CK(19))
    pr[16] = (K("d37") * CK(15) * CC(3) + K("d62") * CC(11) * CC(11) + HET(2) * CK(14) * CK(13)
              + HET(5) * CK(15) * CK(13))
    pe[16] = TJ("cl2")
    pr[17] = K("a27") * CC(6) * CC(6)
    pe[17] = TJ("h2o2") + K("a30") * CC(2) + rain_h2o2
    pr[18] = K("d36") * CC(3) * CC(7) + HET(4) * CK(6) * CK(13)
    pe[18] = TJ("clno2")
    pr[19] = K("e7") * CC(6) * CC(9) + K("c19") * CK(28) * CC(9)
    pe[19] = (K("e11") * CC(2) + K("e9") * CC(1) + TJ("hbr")) * parthbr + HET(8) * CK(26) + HET(9) * CK(15) + rain_hbr
    pr[20] = K("e13") * CC(12) * CC(7)
    pe[20] = TJ("brono2") + K("e8") * CC(4) + HET(6) * CK(3)
    pr[21] = ((TJ("hno4") + K("b28") * CC(2) + K("b24") * hnm) * CK(22) + TJ("hno3") * CK(5) * parthno3
              + 2 * (TJ("n2o5") + K("b32") * hnm) * CK(6) + 2 * K("b39") * CC(1) * CK(1) + TJ("clno2") * CK(18)
              + K("b27") * CK(5) * parthno3 * CC(2) + K("d32") * CK(14) * CC(4)
              + (TJ("clono2_cl") + TJ("clono2_clo")) * CK(14) + TJ("brono2") * CK(20) + K("e8") * CK(20) * CC(4))
    fam[21] = ((K("d31") * CC(11) + K("b22") * CC(2) + K("b23") * CC(6) + 2 * K("b12") * CC(13) + K("d36") * CC(3)
                + K("e13") * CC(12)) * CC(7) + 2 * K("b6") * CC(10) * CC(8))
    pr[22] = K("b23") * CC(6) * CC(7)
    pe[22] = TJ("hno4") + K("b28") * CC(2) + K("b24") * hnm + rain_hno4
    pr[23] = (2 * (K("d61") * hnm + TJ("cl2o2")) * CK(25)
              + (TJ("clono2_cl") + TJ("clono2_clo") + K("d32") * CC(4)) * CK(14)
              + (TJ("hocl") + K("d34") * CC(2) + K("d35") * CC(4)) * CK(15)
              + TJ("oclo") * CK(10) + (TJ("hcl") + K("d11") * CC(2)) * CK(13) * parthcl
              + 2 * TJ("cl2") * CK(16) + TJ("clno2") * CK(18) + TJ("brcl") * CK(27)
              + 3 * (TJ("cfc11") + K("d90") * CC(1)) * CK(31) + 2 * (TJ("cfc12") + K("d91") * CC(1)) * CK(32)
              + 3 * (TJ("cfc113") + K("d92") * CC(1)) * CK(33) + 4 * (TJ("ccl4") + K("d93") * CC(1)) * CK(34)
              + 3 * (TJ("ch3ccl3") + K("d94") * CC(2)) * CK(35) + (TJ("ch3cl") + K("d95") * CC(2)) * CK(36)
              + (TJ("hcfc22") + K("d96") * CC(1) + K("d97") * CC(2)) * CK(37))
    fam[23] = ((K("d31") * CC(7) + 2 * K("d60") * CC(11) + 2 * K("d62") * CC(11) + K("e5a") * CC(12)
                + K("e5c") * CC(12) + K("d9") * CC(2) + K("d33") * CC(6)) * CC(11)
               + (K("c10") * CK(28) + K("d5") * CK(2) + K("d7") * CC(6) + K("d6") * h2 + K("d36") * CC(7)
                  + K("d37") * CK(15)) * CC(3))
    pr[24] = (TJ("hobr") * CK(26) + TJ("brono2") * CK(20) + K("e8") * CK(20) * CC(4) + K("e16") * CK(26) * CC(4)
              + TJ("brcl") * CK(27) + (K("e11") * CC(2) + K("e9") * CC(1) + TJ("hbr")) * CK(19) * parthbr
              + 2 * HET(8) * CK(19) * CK(26))
    fam[24] = ((K("e13") * CC(7) + K("e5c") * CC(11) + K("e15") * CC(6)) * CC(12) + K("c19") * CC(9) * CK(28)
               + K("e7") * CC(9) * CC(6))
    pr[25] = K("d60") * CC(11) * CC(11)
    pe[25] = TJ("cl2o2") + K("d61") * hnm
    pr[26] = K("e15") * CC(12) * CC(6) + HET(6) * CK(20) * CK(3)
    pe[26] = TJ("hobr") + K("e16") * CC(4) + HET(7) * CK(13) + HET(8) * CK(19)
    pr[27] = K("e5c") * CC(11) * CC(12) + HET(7) * CK(26) * CK(13) + HET(9) * CK(19) * CK(15)
    pe[27] = TJ("brcl")
    pr[28] = K("c1c") * CC(1) * CK(2) + K("c3") * CC(4) * CC(15) + K("c15") * ch3o * o2 + K("c17b") * CC(2) * CK(30)
    pe[28] = (K("c8") * CC(2) + K("c9") * CC(4) + K("c10") * CC(3) + K("c19") * CC(9) + TJ("ch2o_hco")
              + TJ("ch2o_co") + rain_ch2o)
    pr[29] = K("c4") * CC(15) * o2 + K("c17a") * CC(2) * CK(30)
    pe[29] = 2 * K("c14") * CK(29) + K("c7") * CC(6) + K("c5") * CC(8) + K("c18") * CC(11)
    pr[30] = K("c7") * CK(29) * CC(6)
    pe[30] = K("c17a") * CC(2) + K("c17b") * CC(2) + TJ("ch3o2h") + rain_ch3o2h
    for n, (j, r) in zip(range(31, 41), [("cfc11", "d90"), ("cfc12", "d91"), ("cfc113", "d92"), ("ccl4", "d93"),
                                          ("ch3ccl3", None), ("ch3cl", None), ("hcfc22", None), ("ch3br", None),
                                          ("h1211", "e52"), ("h1301", "e53")]):
        pr[n] = 0
    pe[31] = TJ("cfc11") + K("d90") * CC(1)
    pe[32] = TJ("cfc12") + K("d91") * CC(1)
    pe[33] = TJ("cfc113") + K("d92") * CC(1)
    pe[34] = TJ("ccl4") + K("d93") * CC(1)
    pe[35] = TJ("ch3ccl3") + K("d94") * CC(2)
    pe[36] = TJ("ch3cl") + K("d95") * CC(2)
    pe[37] = TJ("hcfc22") + K("d96") * CC(1) + K("d97") * CC(2)
    pe[38] = TJ("ch3br") + K("e50") * CC(1) + K("e51") * CC(2)
    pe[39] = TJ("h1211") + K("e52") * CC(1)
    pe[40] = TJ("h1301") + K("e53") * CC(1)
    pr[41] = ((TJ("ch3br") + K("e50") * CC(1) + K("e51") * CC(2)) * CK(38) + (TJ("h1211") + K("e52") * CC(1)) * CK(39)
              + (TJ("h1301") + K("e53") * CC(1)) * CK(40) + 2 * (K("e54") * CC(2) + TJ("ch2br2")) * CK(42))
    fam[41] = rain_hbr * CK(19)
    pr[42] = 0
    pe[42] = TJ("ch2br2") + K("e54") * CC(2)

    res = [None] * NX
    for n in range(1, NL + 1):
        if n in fam:
            res[n - 1] = CK(n) + dt * fam[n] - CK0[n - 1] - dt * pr[n]
        else:
            res[n - 1] = CK(n) * (1 + dt * pe[n]) - CK0[n - 1] - dt * pr[n]
    for s in range(1, NS + 1):
        res[NL + s - 1] = CC(s) - g[s]
    return m, [sp.sympify(r) for r in res]


# --------------------------------------------------------------------------- #
# code emission
# --------------------------------------------------------------------------- #
class Printer(C99CodePrinter):
    """Numbers as T(...) so that the float instantiation stays in FP32;
    integer powers as products."""

    def __init__(self, real="T"):
        super().__init__()
        self.real = real

    def _print_Float(self, e):
        return f"{self.real}({repr(float(e))})"

    def _print_Integer(self, e):
        return f"{self.real}({int(e)})"

    def _print_Rational(self, e):
        return f"{self.real}({float(e)!r})"

    def _print_Pow(self, e):
        b, ex = e.args
        if ex == sp.Rational(1, 2):
            return f"sqrt({self._print(b)})"
        if ex == -1:
            return f"({self.real}(1)/({self._print(b)}))"
        if ex.is_Integer and 0 < ex <= 4:
            s = self.parenthesize(b, 100)
            return "(" + "*".join([s] * int(ex)) + ")"
        if ex.is_Integer and -4 <= ex < 0:
            s = self.parenthesize(b, 100)
            return f"({self.real}(1)/({'*'.join([s] * int(-ex))}))"
        if ex == sp.Rational(-1, 2):
            return f"({self.real}(1)/sqrt({self._print(b)}))"
        if ex == sp.Rational(-3, 2):
            return f"({self.real}(1)/(({self._print(b)})*sqrt({self._print(b)})))"
        raise ValueError(f"unexpected power {e}")

    def _print_Max(self, e):
        a, b = e.args
        return f"fmax({self._print(a)}, {self._print(b)})"

    def _print_Symbol(self, e):
        return e.name


def emit_values(m, res, P, cast_x):
    lines = []
    for kind, s, payload, g in m.stmts:
        if kind == "let":
            lines.append(f"    const T {s.name} = {P.doprint(payload)};")
        elif kind == "sel":
            lhs, rhs, a, b = payload
            lines.append(f"    const T {s.name} = ({P.doprint(lhs)}) > ({P.doprint(rhs)}) ? T({P.doprint(a)}) : "
                         f"T({P.doprint(b)});")
        else:
            a, b = payload
            fn = "fmin" if kind == "min" else "fmax"
            lines.append(f"    const T {s.name} = {fn}({P.doprint(a)}, {P.doprint(b)});")
    return lines


def emit_jacobian(m, res, P, slot):
    lines = []
    for kind, s, payload, g in m.stmts:
        if kind == "let":
            lines.append(f"    const T {s.name} = {P.doprint(payload)};")
            for j, e in sorted(g.items()):
                lines.append(f"    const T d_{s.name}_{j} = {P.doprint(e)};")
        elif kind == "sel":
            lhs, rhs, a, b = payload
            lines.append(f"    const bool sel_{s.name} = ({P.doprint(lhs)}) > ({P.doprint(rhs)});")
            lines.append(f"    const T {s.name} = sel_{s.name} ? T({P.doprint(a)}) : T({P.doprint(b)});")
            for j, (ga, gb) in sorted(g.items()):
                lines.append(f"    const T d_{s.name}_{j} = sel_{s.name} ? T({P.doprint(ga)}) : T({P.doprint(gb)});")
        else:
            a, b = payload
            fn, cmp = ("fmin", "<=") if kind == "min" else ("fmax", ">=")
            lines.append(f"    const T {s.name} = {fn}({P.doprint(a)}, {P.doprint(b)});")
            lines.append(f"    const bool sel_{s.name} = ({P.doprint(a)}) {cmp} ({P.doprint(b)});")
            for j, (ga, gb) in sorted(g.items()):
                lines.append(f"    const T d_{s.name}_{j} = sel_{s.name} ? T({P.doprint(ga)}) : T({P.doprint(gb)});")
    pattern = {}
    for i, r in enumerate(res):
        gr = m.gradient(r)
        for j, e in sorted(gr.items()):
            pattern[(i, j)] = e
    return lines, pattern


def min_degree_order(nz, n):
    """Minimum-degree ordering of the symmetrised pattern."""
    adj = {i: set() for i in range(n)}
    for (i, j) in nz:
        if i != j:
            adj[i].add(j)
            adj[j].add(i)
    order, left = [], set(range(n))
    while left:
        v = min(left, key=lambda u: (len(adj[u] & left), u))
        order.append(v)
        nb = adj[v] & left
        for a in nb:
            adj[a] |= nb - {a}
        left.remove(v)
    return order


def lu_pattern(nz, perm, n):
    """Fill pattern of LU without pivoting in the permuted order."""
    pos = {v: k for k, v in enumerate(perm)}
    rows = [set() for _ in range(n)]
    for (i, j) in nz:
        rows[pos[i]].add(pos[j])
    for k in range(n):
        rows[k].add(k)
    for k in range(n):
        for i in range(k + 1, n):
            if k in rows[i]:
                rows[i] |= {j for j in rows[k] if j > k}
    return rows


def generate(path):
    md, rd = build(True)
    mn, rn = build(False)
    P = Printer("T")
    jd_lines, pat_d = emit_jacobian(md, rd, P, None)
    jn_lines, pat_n = emit_jacobian(mn, rn, P, None)
    nz = set(pat_d) | set(pat_n) | {(i, i) for i in range(NX)}
    perm = min_degree_order(nz, NX)
    rows = lu_pattern(nz, perm, NX)
    slots = {}
    for k in range(NX):
        for j in sorted(rows[k]):
            slots[(k, j)] = len(slots)
    nslot = len(slots)
    pos = {v: k for k, v in enumerate(perm)}
    nnz_orig = len(nz)

    out = []
    w = out.append
    w("// newton_gen.cuh — GENERATED by reprobus_gb300/codegen/gen_newton.py; do not edit.")
    w("//")
    w("// Residual, analytic Jacobian and sparse LU of the chemistry step equations")
    w("// (fixed point of one pass of src/reprobus_l137_20230723.f:1350-2372, in the")
    w("// Jacobi form described in the generator). Unknowns x[0..41] = ck(1..42),")
    w("// x[42..56] = cc(1..15).")
    w(f"// Jacobian: {nnz_orig} structural non-zeros (day|night|diagonal); LU slots with fill: {nslot};")
    w(f"// minimum-degree order: {perm}")
    w("#pragma once")
    w("#ifndef __CUDACC__")
    w("#define __device__")
    w("#define __forceinline__ inline")
    w("#define NT_FN inline")
    w("#else")
    w("#define NT_FN __noinline__  // each generated block gets its own register allocation")
    w("#endif")
    w("")
    w("namespace rpb {")
    w(f"constexpr int NT_NX = {NX};")
    w(f"constexpr int NT_NSLOT = {nslot};")
    w(f"constexpr int NT_NNZ = {nnz_orig};")
    w(f"constexpr int NT_PERM[{NX}] = {{{', '.join(map(str, perm))}}};  // LU position k holds unknown NT_PERM[k]")
    inv = {v: k for k, v in slots.items()}
    w(f"constexpr int NT_SLOT_I[{nslot}] = {{{', '.join(str(perm[inv[s][0]]) for s in range(nslot))}}};")
    w(f"constexpr int NT_SLOT_J[{nslot}] = {{{', '.join(str(perm[inv[s][1]]) for s in range(nslot))}}};")
    w("")
    w("// per-cell constants of the equations")
    w("struct NtFix {")
    w("    double o2, n2, h2, co2, hnm, parthno3, parth2o, parthcl, parthbr;")
    w("    double rain_hno3, rain_hcl, rain_hbr, rain_h2o2, dt;")
    w("};")
    w("template <typename T> struct NtFixT {")
    w("    T o2, n2, h2, co2, hnm, parthno3, parth2o, parthcl, parthbr;")
    w("    T rain_hno3, rain_hcl, rain_hbr, rain_h2o2, dt;")
    w("};")
    for tag, m, res in (("day", md, rd), ("night", mn, rn)):
        w("")
        w(f"// residual R(x), {tag} equations (PK/PX/PR: pointers or strided views)")
        w(f"template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>")
        w(f"__device__ NT_FN void nt_residual_{tag}(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {{")
        out.extend(emit_values(m, res, P, None))
        for i, r in enumerate(res):
            w(f"    R[{i}] = {P.doprint(r)};")
        w("}")
        w("")
        lines, pat = (jd_lines, pat_d) if tag == "day" else (jn_lines, pat_n)
        w(f"// Jacobian dR/dx, {tag} equations, into the LU slots (T = double or float)")
        w(f"template <typename T, typename FF, typename PK, typename PX, typename PJ>")
        w(f"__device__ NT_FN void nt_jacobian_{tag}(const FF& F, PK K, PK tj, PK het, PX x, PJ J) {{")
        out.extend(lines)
        filled = set()
        for (i, j), e in sorted(pat.items()):
            sl = slots[(pos[i], pos[j])]
            filled.add(sl)
            w(f"    J[{sl}] = {P.doprint(e)};")
        for sl in range(nslot):
            if sl not in filled:
                w(f"    J[{sl}] = T(0);")
        w("}")
    # scaling to relative units J'_ij = J_ij * s_j / s_i (s, rs = 1/s in original numbering)
    w("")
    w("template <typename T, typename PJ>")
    w("__device__ NT_FN void nt_scale(PJ J, const T* __restrict__ s, const T* __restrict__ rs) {")
    for (k, j), sl in sorted(slots.items(), key=lambda kv: kv[1]):
        w(f"    J[{sl}] *= s[{perm[j]}] * rs[{perm[k]}];")
    w("}")
    # LU factorisation and solve (permuted order; b in original numbering)
    w("")
    w("// in-place LU (no pivoting) of the permuted sparse matrix; a zero or")
    w("// non-finite pivot is replaced by tiny (the FP64 residual corrects the step)")
    w("template <typename T, typename PJ>")
    w("__device__ NT_FN void nt_lu(PJ J, T tiny) {")
    for k in range(NX):
        dk = slots[(k, k)]
        w(f"    {{ T p = J[{dk}]; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny; J[{dk}] = p; const T r = T(1) / p;")
        for i in range(k + 1, NX):
            if (i, k) in slots:
                lik = slots[(i, k)]
                w(f"      {{ const T l = J[{lik}] * r; J[{lik}] = l;")
                for j in sorted(rows[k]):
                    if j > k:
                        w(f"        J[{slots[(i, j)]}] -= l * J[{slots[(k, j)]}];")
                w("      }")
        w("    }")
    w("}")
    w("")
    w("// solve (LU) y = b; b is given and returned in the original numbering")
    w("template <typename T, typename PJ>")
    w("__device__ NT_FN void nt_solve(PJ J, T* __restrict__ b) {")
    w(f"    T y[{NX}];")
    for k in range(NX):
        terms = [f" - J[{slots[(k, j)]}] * y[{j}]" for j in sorted(rows[k]) if j < k]
        w(f"    y[{k}] = b[{perm[k]}]{''.join(terms)};")
    for k in range(NX - 1, -1, -1):
        terms = [f" - J[{slots[(k, j)]}] * y[{j}]" for j in sorted(rows[k]) if j > k]
        w(f"    y[{k}] = (y[{k}]{''.join(terms)}) / J[{slots[(k, k)]}];")
    for k in range(NX):
        w(f"    b[{perm[k]}] = y[{k}];")
    w("}")
    w("}  // namespace rpb")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return {"nnz": nnz_orig, "slots": nslot, "perm": perm}


if __name__ == "__main__":
    target = os.path.join(os.path.dirname(HERE), "csrc", "newton_gen.cuh")
    info = generate(target)
    print(f"wrote {target}: nnz {info['nnz']}, LU slots {info['slots']}")
