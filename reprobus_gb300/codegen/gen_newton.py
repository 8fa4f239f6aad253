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
    integer powers as products; every quotient as nt_div<T>(numerator,
    denominator) (newton_num.cuh)."""

    def __init__(self, real="T"):
        super().__init__()
        self.real = real

    def _print_Float(self, e):
        return f"{self.real}({repr(float(e))})"

    def _print_Integer(self, e):
        return f"{self.real}({int(e)})"

    def _print_Rational(self, e):
        return f"{self.real}({float(e)!r})"

    def _div(self, num, den):
        return f"nt_div<{self.real}>({num}, {den})"

    def _print_Mul(self, e):
        num, den = sp.fraction(e, exact=True)
        if den == 1:
            return super()._print_Mul(e)
        return self._div(self._print(num), self._print(den))

    def _print_Pow(self, e):
        b, ex = e.args
        if ex == sp.Rational(1, 2):
            return f"sqrt({self._print(b)})"
        if ex == -1:
            return self._div(f"{self.real}(1)", self._print(b))
        if ex.is_Integer and 0 < ex <= 4:
            s = self.parenthesize(b, 100)
            return "(" + "*".join([s] * int(ex)) + ")"
        if ex.is_Integer and -4 <= ex < 0:
            s = self.parenthesize(b, 100)
            return self._div(f"{self.real}(1)", "*".join([s] * int(-ex)))
        if ex == sp.Rational(-1, 2):
            return self._div(f"{self.real}(1)", f"sqrt({self._print(b)})")
        if ex == sp.Rational(-3, 2):
            return self._div(f"{self.real}(1)", f"({self._print(b)})*sqrt({self._print(b)})")
        raise ValueError(f"unexpected power {e}")

    def _print_Max(self, e):
        a, b = e.args
        return f"fmax({self._print(a)}, {self._print(b)})"

    def _print_Symbol(self, e):
        return e.name


class XPrinter(Printer):
    """Jacobian printer: the FP64 iterate x[j] is read once per call, rounded
    to T (xt{j}, defined at the top of the function)."""

    def _print_Symbol(self, e):
        n = e.name
        if n.startswith("x["):
            return f"xt{n[2:-1]}"
        return n


def _cse(exprs, prefix, P, real="T"):
    """sympy CSE of a list of expressions -> (definition lines, reduced list)."""
    rep, red = sp.cse(exprs, symbols=sp.numbered_symbols(prefix))
    return [f"    const {real} {s.name} = {P.doprint(e)};" for s, e in rep], red


def emit_statements(m, P, derivs):
    """The named intermediates (and, with derivs, their gradients), one chunk
    of lines per statement, with common subexpressions (shared reciprocals
    above all) evaluated once."""
    chunks = []
    for idx, (kind, s, payload, g) in enumerate(m.stmts):
        lines = []
        pre = f"{s.name}_c"
        keys = sorted(g) if derivs else []
        if kind == "let":
            defs, red = _cse([payload] + [g[j] for j in keys], pre, P)
            lines += defs
            lines.append(f"    const T {s.name} = {P.doprint(red[0])};")
            for j, e in zip(keys, red[1:]):
                lines.append(f"    const T d_{s.name}_{j} = {P.doprint(e)};")
            chunks.append(lines)
            continue
        if kind == "sel":
            lhs, rhs, a, b = payload
            cond = (lhs, rhs, ">")
        else:
            a, b = payload
            cond = (a, b, "<=" if kind == "min" else ">=")
        exprs = [cond[0], cond[1], a, b] + [g[j][0] for j in keys] + [g[j][1] for j in keys]
        defs, red = _cse(exprs, pre, P)
        lines += defs
        c0, c1, ra, rb = (P.doprint(e) for e in red[:4])
        lines.append(f"    const bool sel_{s.name} = ({c0}) {cond[2]} ({c1});")
        lines.append(f"    const T {s.name} = sel_{s.name} ? T({ra}) : T({rb});")
        nk = len(keys)
        for q, j in enumerate(keys):
            ga, gb = P.doprint(red[4 + q]), P.doprint(red[4 + nk + q])
            lines.append(f"    const T d_{s.name}_{j} = sel_{s.name} ? T({ga}) : T({gb});")
        chunks.append(lines)
    return chunks


def ready_after(m, exprs):
    """Index of the last statement whose value or gradient symbols the
    expressions use (-1: none), so that each row is emitted as soon as it
    can be and the intermediates it reads die early."""
    names = {}
    for idx, (_, s, _, g) in enumerate(m.stmts):
        names[s.name] = idx
        for j in g:
            names[f"d_{s.name}_{j}"] = idx
    last = -1
    for e in exprs:
        for u in sp.sympify(e).free_symbols:
            if u.name in names:
                last = max(last, names[u.name])
    return last


def jacobian_entries(m, res):
    """(i, j) -> dR_i/dx_j in terms of the intermediates' gradient symbols."""
    pattern = {}
    for i, r in enumerate(res):
        for j, e in sorted(m.gradient(r).items()):
            pattern[(i, j)] = e
    return pattern


# --------------------------------------------------------------------------- #
# elimination order and storage plan
# --------------------------------------------------------------------------- #
def filled_rows(nz, perm, n):
    """Rows (in elimination positions) of the LU fill pattern without pivoting."""
    pos = {v: k for k, v in enumerate(perm)}
    rows = [set() for _ in range(n)]
    for (i, j) in nz:
        rows[pos[i]].add(pos[j])
    for k in range(n):
        rows[k].add(k)
    for k in range(n):
        rk = [j for j in rows[k] if j > k]
        for i in range(k + 1, n):
            if k in rows[i]:
                rows[i].update(rk)
    return rows


def lu_updates(rows, n):
    return sum(sum(1 for j in rows[k] if j > k) for i in range(n) for k in rows[i] if k < i)


def markowitz_order(nz, n):
    """Diagonal Markowitz ordering: eliminate next the unknown whose pivot has
    the fewest (row count - 1)(column count - 1) in the active submatrix."""
    R = {i: set() for i in range(n)}
    C = {j: set() for j in range(n)}
    for (i, j) in nz:
        R[i].add(j)
        C[j].add(i)
    left, order = set(range(n)), []
    while left:
        def key(v):
            r = len(R[v] & left) - 1
            c = len(C[v] & left) - 1
            return (r * c, r + c, v)
        v = min(left, key=key)
        order.append(v)
        rs, cs = R[v] & left, C[v] & left
        for i in cs - {v}:
            for j in rs - {v}:
                R[i].add(j)
                C[j].add(i)
        left.remove(v)
    return order


def refine_order(nz, n, perm, iters=4000, seed=1):
    """Deterministic local search (move one unknown) that keeps any move which
    does not increase the LU update count."""
    import random
    rnd = random.Random(seed)
    cur = list(perm)
    cost = lu_updates(filled_rows(nz, cur, n), n)
    for _ in range(iters):
        a, b = rnd.randrange(n), rnd.randrange(n)
        if a == b:
            continue
        o = cur[:]
        o.insert(b, o.pop(a))
        c = lu_updates(filled_rows(nz, o, n), n)
        if c <= cost:
            cur, cost = o, c
    return cur


def storage_plan(nz, const, perm, rows, n):
    """Shared-memory slots of one cell. The Jacobian writes every stored entry
    of A (constant diagonal entries are not stored); row t of the row-by-row
    (Crout) factorisation reads its A entries into registers and writes the
    off-diagonal entries of the unit upper factor U~ into slots freed by rows
    <= t (lowest free slot first), so the peak is what the plan needs."""
    import heapq
    pos = {v: k for k, v in enumerate(perm)}
    arow = [[] for _ in range(n)]
    for (i, j) in nz:
        if (i, j) not in const:
            arow[pos[i]].append(pos[j])
    slot_a = {}
    for t in range(n):
        for c in sorted(arow[t]):
            slot_a[(t, c)] = len(slot_a)
    na = len(slot_a)
    free, nxt, slot_u = [], na, {}
    for t in range(n):
        for c in arow[t]:
            heapq.heappush(free, slot_a[(t, c)])
        for j in sorted(c for c in rows[t] if c > t):
            if free:
                slot_u[(t, j)] = heapq.heappop(free)
            else:
                slot_u[(t, j)] = nxt
                nxt += 1
    return slot_a, slot_u, na, max(na, nxt)


# --------------------------------------------------------------------------- #
# emission
# --------------------------------------------------------------------------- #
def emit_residual(w, tag, m, res, P):
    w("")
    w(f"// residual R(x), {tag} equations (FP64; K/tj/het/ck0/x: pointers or views)")
    w("template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>")
    w(f"__device__ __forceinline__ void nt_residual_{tag}(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {{")
    chunks = emit_statements(m, P, derivs=False)
    at = {}
    for i, r in enumerate(res):
        at.setdefault(ready_after(m, [r]), []).append(i)
    for idx in range(-1, len(chunks)):
        if idx >= 0:
            for line in chunks[idx]:
                w(line)
        for i in at.get(idx, []):
            defs, red = _cse([res[i]], f"{tag[0]}r{i}_c", P)
            for line in defs:
                w(line)
            w(f"    R[{i}] = {P.doprint(red[0])};")
    w("}")


def emit_jacobian(w, tag, m, pat, union, const, slot_a, pos, XP):
    w("")
    w(f"// scaled Jacobian J'_ij = dR_i/dx_j s_j / s_i, {tag} equations, into the")
    w("// stored A slots (T = double or float; x: FP64 iterate; s: nt_exp_hi scales)")
    w("template <typename T, typename FF, typename PK, typename PJ>")
    w(f"__device__ __forceinline__ void nt_jacobian_{tag}(const FF& F, PK K, PK tj, PK het, "
      "const double* __restrict__ x, double floor_, PJ J) {")
    w("    const int fh = nt_exp_hi(floor_);")
    w("    // the iterate in T and the column scales, once per call")
    for j in range(NX):
        w(f"    const T xt{j} = nt_cvt<T>(x[{j}]);")
    for j in range(NX):
        w(f"    const T cs{j} = nt_scale<T>(nt_exp_hi(x[{j}]), fh);")
    chunks = emit_statements(m, XP, derivs=True)
    by_row = {}
    for (i, j) in sorted(union):
        by_row.setdefault(i, []).append(j)
    at = {}
    for i in range(NX):
        cols = by_row.get(i, [])
        exprs = [pat.get((i, j), sp.Integer(0)) for j in cols]
        at.setdefault(ready_after(m, exprs), []).append(i)
        for j in cols:
            if (i, j) in const:
                v = pat.get((i, j), sp.Integer(0))
                assert v == const[(i, j)], ((i, j), v)
    for idx in range(-1, len(chunks)):
        if idx >= 0:
            for line in chunks[idx]:
                w(line)
        for i in at.get(idx, []):
            stored = [j for j in by_row.get(i, []) if (i, j) not in const]
            exprs = [pat.get((i, j), sp.Integer(0)) for j in stored]
            defs, red = _cse(exprs, f"{tag[0]}j{i}_c", XP)
            w(f"    {{  // row {i}")
            w(f"    const T rs{i} = nt_rscale<T>(nt_exp_hi(x[{i}]), fh);")
            for line in defs:
                w("    " + line)
            for j, e in zip(stored, red):
                sl = slot_a[(pos[i], pos[j])]
                if e == 0:
                    w(f"        J[{sl}] = T(0);")
                else:
                    w(f"        J[{sl}] = ({XP.doprint(e)}) * (cs{j} * rs{i});")
            w("    }")
    w("}")


# --------------------------------------------------------------------------- #
# row groups: the residual and Jacobian rows split among W warps that work on
# the same cells, each group with the intermediates its rows need
# --------------------------------------------------------------------------- #
def stmt_symbols(m):
    """name -> statement index for every value and gradient symbol."""
    names = {}
    for idx, (_, s, _, g) in enumerate(m.stmts):
        names[s.name] = idx
        for j in g:
            names[f"d_{s.name}_{j}"] = idx
    return names


def stmt_refs(m, derivs):
    """Per statement, the statements its value (and, with derivs, its
    gradient) reads."""
    names = stmt_symbols(m)
    out = []
    for idx, (kind, s, payload, g) in enumerate(m.stmts):
        exprs = list(payload) if isinstance(payload, tuple) else [payload]
        if derivs:
            for j, e in g.items():
                if e is None:
                    continue
                exprs += list(e) if isinstance(e, tuple) else [e]
        if derivs and kind != "let":
            # min/max/sel gradients are emitted from the branches' gradients
            for u in payload:
                exprs += list(m.gradient(sp.sympify(u)).values())
        refs = set()
        for e in exprs:
            for u in sp.sympify(e).free_symbols:
                if u.name in names and names[u.name] != idx:
                    refs.add(names[u.name])
        out.append(refs)
    return out


def closure(m, exprs, refs):
    """Indices of the statements the expressions need, transitively."""
    names = stmt_symbols(m)
    need, todo = set(), []
    for e in exprs:
        for u in sp.sympify(e).free_symbols:
            if u.name in names:
                todo.append(names[u.name])
    while todo:
        i = todo.pop()
        if i in need:
            continue
        need.add(i)
        todo.extend(refs[i])
    return need


def stmt_cost(m, derivs):
    out = []
    for kind, s, payload, g in m.stmts:
        exprs = list(payload) if isinstance(payload, tuple) else [payload]
        if derivs:
            for e in g.values():
                if e is not None:
                    exprs += list(e) if isinstance(e, tuple) else [e]
        out.append(sum(sp.count_ops(sp.sympify(e)) for e in exprs) + 1)
    return out


def partition_rows(m, row_exprs, W, derivs):
    """Rows (index -> list of expressions) split into W groups of balanced
    cost (operations of the rows plus those of the statements each group
    evaluates, shared statements counted once per group that needs them)."""
    refs = stmt_refs(m, derivs)
    scost = stmt_cost(m, derivs)
    info = {}
    for i, exprs in row_exprs.items():
        info[i] = (sum(sp.count_ops(sp.sympify(e)) for e in exprs) + 1, closure(m, exprs, refs))
    groups = [[] for _ in range(W)]
    have = [set() for _ in range(W)]
    cost = [0] * W
    for i in sorted(info, key=lambda r: -(info[r][0] + sum(scost[k] for k in info[r][1]))):
        rc, need = info[i]
        best = min(range(W), key=lambda g: (cost[g] + rc + sum(scost[k] for k in need - have[g]), g))
        groups[best].append(i)
        cost[best] += rc + sum(scost[k] for k in need - have[best])
        have[best] |= need
    return [sorted(g) for g in groups], cost, [sorted(h) for h in have]


def emit_residual_group(w, tag, m, res, P, rows, name):
    need = closure(m, [res[i] for i in rows], stmt_refs(m, False))
    w("")
    w(f"// residual rows {rows} ({tag} equations, FP64)")
    w("template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>")
    w(f"__device__ __forceinline__ void {name}(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {{")
    chunks = emit_statements(m, P, derivs=False)
    at = {}
    for i in rows:
        at.setdefault(ready_after(m, [res[i]]), []).append(i)
    for idx in range(-1, len(chunks)):
        if idx >= 0 and idx in need:
            for line in chunks[idx]:
                w(line)
        for i in at.get(idx, []):
            defs, red = _cse([res[i]], f"{tag[0]}r{i}_c", P)
            for line in defs:
                w(line)
            w(f"    R[{i}] = {P.doprint(red[0])};")
    w("}")


def emit_jacobian_group(w, tag, m, pat, union, const, slot_a, pos, XP, rows, name):
    by_row = {}
    for (i, j) in sorted(union):
        by_row.setdefault(i, []).append(j)
    row_exprs = {i: [pat.get((i, j), sp.Integer(0)) for j in by_row.get(i, []) if (i, j) not in const] for i in rows}
    need = closure(m, [e for es in row_exprs.values() for e in es], stmt_refs(m, True))
    w("")
    w(f"// scaled Jacobian rows {rows} ({tag} equations) into their stored A slots")
    w("template <typename T, typename FF, typename PK, typename PJ>")
    w(f"__device__ __forceinline__ void {name}(const FF& F, PK K, PK tj, PK het, "
      "const double* __restrict__ x, double floor_, PJ J) {")
    w("    const int fh = nt_exp_hi(floor_);")
    for j in range(NX):
        w(f"    const T xt{j} = nt_cvt<T>(x[{j}]);")
    for j in sorted({j for i in rows for j in by_row.get(i, []) if (i, j) not in const}):
        w(f"    const T cs{j} = nt_scale<T>(nt_exp_hi(x[{j}]), fh);")
    chunks = emit_statements(m, XP, derivs=True)
    at = {}
    for i in rows:
        at.setdefault(ready_after(m, row_exprs[i]), []).append(i)
    for idx in range(-1, len(chunks)):
        if idx >= 0 and idx in need:
            for line in chunks[idx]:
                w(line)
        for i in at.get(idx, []):
            stored = [j for j in by_row.get(i, []) if (i, j) not in const]
            if not stored:
                continue
            defs, red = _cse([pat.get((i, j), sp.Integer(0)) for j in stored], f"{tag[0]}j{i}_c", XP)
            w(f"    {{  // row {i}")
            w(f"    const T rs{i} = nt_rscale<T>(nt_exp_hi(x[{i}]), fh);")
            for line in defs:
                w("    " + line)
            for j, e in zip(stored, red):
                sl = slot_a[(pos[i], pos[j])]
                if e == 0:
                    w(f"        J[{sl}] = T(0);")
                else:
                    w(f"        J[{sl}] = ({XP.doprint(e)}) * (cs{j} * rs{i});")
            w("    }")
    w("}")


def emit_groups(w, W, tag, m, res, pat, union, const, slot_a, pos, P, XP, stats):
    """W residual and W Jacobian row groups of the day or night equations and
    their dispatchers (g: the group, warp-uniform)."""
    by_row = {}
    for (i, j) in sorted(union):
        by_row.setdefault(i, []).append(j)
    rgroups, rcost, _ = partition_rows(m, {i: [res[i]] for i in range(NX)}, W, False)
    jrows = {i: [pat.get((i, j), sp.Integer(0)) for j in by_row.get(i, []) if (i, j) not in const]
             for i in range(NX)}
    jrows = {i: e for i, e in jrows.items() if e}
    jgroups, jcost, _ = partition_rows(m, jrows, W, True)
    stats[(tag, W)] = (rcost, jcost)
    for g in range(W):
        emit_residual_group(w, tag, m, res, P, rgroups[g], f"nt_residual_{tag}_w{W}_{g}")
        emit_jacobian_group(w, tag, m, pat, union, const, slot_a, pos, XP, jgroups[g], f"nt_jacobian_{tag}_w{W}_{g}")
    w("")
    w(f"// residual rows of group g of {W} ({tag} equations)")
    w("template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>")
    w(f"__device__ __forceinline__ void nt_residual_{tag}_w{W}(int g, const FF& F, PK K, PK tj, PK het, PC ck0, PX x, "
      "PR R) {")
    w("    switch (g) {")
    for g in range(W):
        w(f"        case {g}: nt_residual_{tag}_w{W}_{g}<T>(F, K, tj, het, ck0, x, R); break;")
    w("        default: break;")
    w("    }")
    w("}")
    w(f"// Jacobian rows of group g of {W} ({tag} equations)")
    w("template <typename T, typename FF, typename PK, typename PJ>")
    w(f"__device__ __forceinline__ void nt_jacobian_{tag}_w{W}(int g, const FF& F, PK K, PK tj, PK het, "
      "const double* __restrict__ x, double floor_, PJ J) {")
    w("    switch (g) {")
    for g in range(W):
        w(f"        case {g}: nt_jacobian_{tag}_w{W}_{g}<T>(F, K, tj, het, x, floor_, J); break;")
    w("        default: break;")
    w("    }")
    w("}")


WARPS_PER_CELL = (2, 4)  # row groups generated for the warps-per-cell solve kernel


def emit_factor(w, perm, rows, slot_a, slot_u, const_pos, n):
    Z = lambda i: f"z[{i}]"
    w("")
    w("// Crout factorisation, row by row in elimination order, of the stored scaled")
    w("// matrix, with the forward substitution fused: row t is read into registers")
    w("// w, reduced by the earlier unit-upper rows U~(k,:), its pivot p = w_t taken")
    w("// (a zero or non-finite pivot replaced by +-tiny: the FP64 residual corrects")
    w("// the step), z_t = (z_t - sum_k w_k z_k) / p and U~(t,j) = w_j / p stored;")
    w("// then the back substitution. z (original numbering, registers or a view):")
    w("// right-hand side in, solution out. L is never stored. NT_FENCE keeps each")
    w("// row's shared-memory loads in that row (hoisted loads would hold registers).")
    w("template <typename T, typename PJ, typename PZ>")
    w("__device__ __forceinline__ void nt_factor_solve(PJ J, PZ z, T tiny) {")
    for t in range(n):
        w("    NT_FENCE();")
        w(f"    {{  // row {t}: unknown {perm[t]}")
        for c in sorted(rows[t]):
            if (t, c) in slot_a:
                w(f"        T w{c} = J[{slot_a[(t, c)]}];")
            elif c == t and t in const_pos:
                w(f"        T w{c} = T({float(const_pos[t])!r});")
            else:
                w(f"        T w{c} = T(0);")
        w(f"        T zt = {Z(perm[t])};")
        for k in sorted(c for c in rows[t] if c < t):
            w(f"        zt -= w{k} * {Z(perm[k])};")
            for j in sorted(c for c in rows[k] if c > k):
                w(f"        w{j} -= w{k} * J[{slot_u[(k, j)]}];")
        w(f"        T p = w{t}; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;")
        w("        const T d = nt_rcp<T>(p);")
        w(f"        {Z(perm[t])} = zt * d;")
        for j in sorted(c for c in rows[t] if c > t):
            w(f"        J[{slot_u[(t, j)]}] = w{j} * d;")
        w("    }")
    for t in range(n - 1, -1, -1):
        terms = "".join(f" - J[{slot_u[(t, j)]}] * {Z(perm[j])}" for j in sorted(c for c in rows[t] if c > t))
        if terms:
            w("    NT_FENCE();")
            w(f"    {Z(perm[t])} = {Z(perm[t])}{terms};")
    w("}")


def generate(path):
    md, rd = build(True)
    mn, rn = build(False)
    P = Printer("T")
    XP = XPrinter("T")
    pat_d = jacobian_entries(md, rd)
    pat_n = jacobian_entries(mn, rn)
    union = set(pat_d) | set(pat_n)
    nz = union | {(i, i) for i in range(NX)}
    # constant diagonal entries (the same number in the day and night equations)
    const = {}
    for (i, j) in nz:
        a, b = pat_d.get((i, j), sp.Integer(0)), pat_n.get((i, j), sp.Integer(0))
        if i == j and a.is_Number and b.is_Number and a == b and a != 0:
            const[(i, j)] = a
    perm = refine_order(nz, NX, markowitz_order(nz, NX))
    rows = filled_rows(nz, perm, NX)
    pos = {v: k for k, v in enumerate(perm)}
    slot_a, slot_u, na, nslot = storage_plan(nz, const, perm, rows, NX)
    const_pos = {pos[i]: v for (i, _), v in const.items()}
    nupd = lu_updates(rows, NX)
    nu = len(slot_u)

    out = []
    w = out.append
    w("// newton_gen.cuh — GENERATED by reprobus_gb300/codegen/gen_newton.py; do not edit.")
    w("//")
    w("// Residual, scaled analytic Jacobian and sparse Crout LU of the chemistry step")
    w("// equations (fixed point of one pass of src/reprobus_l137_20230723.f:1350-2372,")
    w("// in the Jacobi form described in the generator). Unknowns x[0..41] = ck(1..42),")
    w("// x[42..56] = cc(1..15).")
    w(f"// Jacobian: {len(nz)} structural non-zeros (day|night|diagonal), {len(const)} of them constant")
    w(f"// diagonal entries; stored A entries {na}; off-diagonal U~ entries {nu}; LU updates {nupd};")
    w(f"// shared-memory slots per cell {nslot}.")
    w(f"// elimination order (Markowitz, refined): {perm}")
    w("#pragma once")
    w("#ifndef __CUDACC__")
    w("#define __device__")
    w("#define __forceinline__ inline")
    w("#endif")
    w('#include "newton_num.cuh"')
    w("")
    w("namespace rpb {")
    w(f"constexpr int NT_NX = {NX};")
    w(f"constexpr int NT_NNZ = {len(nz)};")
    w(f"constexpr int NT_NA = {na};        // stored entries of A (the Jacobian)")
    w(f"constexpr int NT_NSLOT = {nslot};     // shared-memory matrix slots per cell")
    w(f"constexpr int NT_NUPD = {nupd};     // multiply-adds of the factorisation")
    w(f"constexpr int NT_PERM[{NX}] = {{{', '.join(map(str, perm))}}};  // elimination position k holds unknown NT_PERM[k]")
    inv_a = {v: k for k, v in slot_a.items()}
    w(f"constexpr int NT_A_I[{na}] = {{{', '.join(str(perm[inv_a[q][0]]) for q in range(na))}}};")
    w(f"constexpr int NT_A_J[{na}] = {{{', '.join(str(perm[inv_a[q][1]]) for q in range(na))}}};")
    ci = sorted(i for (i, _) in const)
    w(f"constexpr int NT_NCONST = {len(ci)};")
    w(f"constexpr int NT_CONST_I[{len(ci)}] = {{{', '.join(map(str, ci))}}};  // constant diagonal entries")
    w(f"constexpr double NT_CONST_V[{len(ci)}] = {{{', '.join(repr(float(const[(i, i)])) for i in ci)}}};")
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
    w("")
    stats = {}
    for tag, m, res, pat in (("day", md, rd, pat_d), ("night", mn, rn, pat_n)):
        emit_residual(w, tag, m, res, P)
        emit_jacobian(w, tag, m, pat, union, const, slot_a, pos, XP)
        for W in WARPS_PER_CELL:
            emit_groups(w, W, tag, m, res, pat, union, const, slot_a, pos, P, XP, stats)
    emit_factor(w, perm, rows, slot_a, slot_u, const_pos, NX)
    w("}  // namespace rpb")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return {"nnz": len(nz), "slots": nslot, "stored": na, "updates": nupd, "perm": perm, "groups": stats}


if __name__ == "__main__":
    target = os.path.join(os.path.dirname(HERE), "csrc", "newton_gen.cuh")
    info = generate(target)
    print(f"wrote {target}: nnz {info['nnz']}, stored A {info['stored']}, slots {info['slots']}, "
          f"LU updates {info['updates']}")
    for (tag, W), (rc, jc) in info["groups"].items():
        print(f"  {tag} W={W}: residual group costs {rc}, Jacobian group costs {jc}")
