"""The C oracle against the golden fixtures of the independent NumPy
restatement (tests/golden/make_golden.py).  CPU only.

Bit-exact where the arithmetic has no transcendental call and no reduction
(level set, Allen-Cahn pre-smoothing, AccDiff, tables, operators, interface
measure, Cahn-Hilliard).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import sbm_oracle as orc

G = np.load(Path(__file__).resolve().parent / "golden" / "golden_v1.npz")


def test_redist_matches_golden():
    sg = G["redist_sg"]
    assert np.array_equal(orc.redist(9, sg, np.zeros_like(sg), 1.0e-1), G["redist_out_d"])
    assert np.array_equal(orc.redist(9, sg, np.zeros_like(sg), float(np.float32(0.1))),
                          G["redist_out_f"])


def test_allen_cahn_matches_golden():
    assert np.array_equal(orc.allen_cahn(17, G["ac_in"]), G["ac_out"])


def test_accdiff_matches_golden():
    psi = G["acc_psi"]
    assert np.array_equal(orc.accdiff(psi, np.zeros_like(psi), 23, 1), G["acc_solid"])
    pe = G["acc_psi_e"]
    assert np.array_equal(orc.accdiff(pe, np.zeros_like(pe), 23, 0), G["acc_elec"])


def test_table_matches_golden():
    assert np.array_equal(orc.table(G["tbl_cord"], G["tbl_vals"], G["tbl_cn"]), G["tbl_out"])


def test_operators_match_golden():
    K, P, psE = G["op_K"], G["op_P"], G["op_psE"]
    dx, dt = float(G["op_dx"]), float(G["op_dt"])
    q = orc.apply(K, P, 1.0 / (dx * dx))
    assert np.array_equal(q[1:-1, 1:-1, 1:-1], G["op_php"])
    q = orc.apply(K * psE, P, dt / (dx * dx), diag=psE)
    assert np.array_equal(q[1:-1, 1:-1, 1:-1], G["op_cne"])


def test_avp_matches_golden():
    psP, psE = G["avp_psP"], G["avp_psE"]
    ny, nx, nz = (s - 2 for s in psP.shape)
    avp = np.zeros(psP.shape, order="F")
    avpx = np.zeros(psP.shape, order="F")
    orc.lib().orc_avp(ny, nx, nz, orc._p(np.asfortranarray(psP)), orc._p(np.asfortranarray(psE)),
                      float(G["op_dx"]), 1.0e-2, orc._p(avp), orc._p(avpx))
    assert np.array_equal(avp[1:-1, 1:-1, 1:-1], G["avp"])
    assert np.array_equal(avpx[1:-1, 1:-1, 1:-1], G["avpx"])


def test_cahn_hilliard_block_matches_golden():
    from elsim_gb300 import sbm
    cnp, psP = G["ch_cnp"], G["ch_psP"]
    ny, nx, nz = (s - 2 for s in cnp.shape)
    p = orc.params_reference()
    p.set_table("tbl_x", G["tbl_cord"])
    p.set_table("tbl_mu", G["ch_mu_t"])
    p.set_table("tbl_mb", G["ch_mb_t"])
    st = orc.State(ny, nx, nz, p)
    st.set_field(sbm.F_CNP, cnp)
    st.set_field(sbm.F_PSP, psP)
    rx = np.zeros_like(cnp)
    rx[1:-1, 1:-1, 1:-1] = G["ch_rxn"]
    ax = np.zeros_like(cnp)
    ax[1:-1, 1:-1, 1:-1] = G["ch_avpx"]
    st.set_field(sbm.F_RXN, rx)
    st.set_field(sbm.F_AVPX, ax)
    dt = float(G["op_dt"])
    # tPP is set by set-up in the program; only Xrf depends on it
    st.ch_step(dt)
    assert np.array_equal(st.field(sbm.F_CNP), G["ch_out"])
