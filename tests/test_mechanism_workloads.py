"""Mechanism generator invariants, generated-code inputs and benchmark workload definitions."""
import numpy as np
import pytest

from pelelm_gb300.mech.generate import DRM19_SPECIES, LIDRYER_SPECIES, generate
from pelelm_gb300.mech.model import Mechanism
from pelelm_gb300.workloads import (CONFIGS, box_layout, from_box_arena, load_mechanism, make_cells,
                                    mech_path, to_box_arena)

SHAPES = {"lidryer_syn": (9, 21), "drm19_syn": (21, 84), "gri_syn": (53, 325)}


@pytest.mark.parametrize("name", list(SHAPES))
def test_shapes_and_element_balance(name):
    m = load_mechanism(name)
    assert (m.ns, m.nr) == SHAPES[name]
    assert m.synthetic
    for r in m.reactions:
        bal = {}
        for side, sign in ((r.reactants, -1), (r.products, 1)):
            for s, nu in side.items():
                for e, n in m.species[m.index(s)].composition.items():
                    bal[e] = bal.get(e, 0) + sign * nu * n
        assert all(v == 0 for v in bal.values()), r.equation()


def test_species_orders_follow_reference_fixtures():
    assert [s.name for s in load_mechanism("lidryer_syn").species] == LIDRYER_SPECIES
    assert [s.name for s in load_mechanism("drm19_syn").species] == DRM19_SPECIES


@pytest.mark.parametrize("name", list(SHAPES))
def test_thermo_continuous_at_tmid(name):
    m = load_mechanism(name)
    for s in m.species:
        T = s.Tmid
        for a_lo, a_hi in ((s.low, s.high),):
            def cp(a):
                return a[0] + a[1] * T + a[2] * T ** 2 + a[3] * T ** 3 + a[4] * T ** 4

            def h(a):
                return a[0] + a[1] * T / 2 + a[2] * T ** 2 / 3 + a[3] * T ** 3 / 4 + a[4] * T ** 4 / 5 + a[5] / T

            def sR(a):
                return a[0] * np.log(T) + a[1] * T + a[2] * T ** 2 / 2 + a[3] * T ** 3 / 3 + a[4] * T ** 4 / 4 + a[6]
            assert abs(cp(a_lo) - cp(a_hi)) < 1e-9 * abs(cp(a_lo))
            assert abs(h(a_lo) - h(a_hi)) < 1e-9 * (abs(h(a_lo)) + 1)
            assert abs(sR(a_lo) - sR(a_hi)) < 1e-9 * (abs(sR(a_lo)) + 1)


def test_generator_is_deterministic(tmp_path):
    a = generate("lidryer_syn")
    p = tmp_path / "x.json"
    a.to_json(str(p))
    b = Mechanism.from_json(str(p))
    committed = load_mechanism("lidryer_syn")
    assert [r.equation() for r in b.reactions] == [r.equation() for r in committed.reactions]
    np.testing.assert_allclose([r.rate.A for r in b.reactions], [r.rate.A for r in committed.reactions])


def test_flat_file_matches_json(tmp_path):
    m = load_mechanism("drm19_syn")
    p = tmp_path / "d.mech"
    m.to_flat(str(p))
    assert p.read_text() == open(mech_path("drm19_syn")).read()


def test_amr_workload_definition():
    cfg = CONFIGS["lidryer_amr120"]
    assert len(cfg.boxes) == 120 and cfg.ncell == 2154496
    assert set(cfg.boxes) == {8, 16, 32, 64}
    assert CONFIGS["lidryer_32cube"].ncell == 32768
    assert CONFIGS["drm19_2M"].ncell == 2 ** 21
    assert CONFIGS["gri_1M"].ncell == 2 ** 20


def test_forcing_is_realizable_and_mass_neutral():
    cfg = CONFIGS["lidryer_amr120"]
    cs = make_cells(cfg, 5000, seed=3)
    assert np.allclose(cs.rYsrc.sum(axis=1), 0.0, atol=1e-12 * np.abs(cs.rYsrc).max())
    assert np.all(cs.rY + cfg.dt * cs.rYsrc >= 0.0)  # species absent at t=0 get no sink
    assert 0.0 < np.std(cs.rYsrc) < 1.0
    assert np.all((cs.T >= 300) & (cs.T <= 2400))


def test_box_arena_roundtrip():
    lay = box_layout([4, 2, 3])
    a = np.random.default_rng(0).normal(size=(lay.ncell, 5))
    np.testing.assert_array_equal(from_box_arena(lay, to_box_arena(lay, a), 5), a)


def test_global_tables_species_reaction_lists_match_stoichiometry():
    """The warp kernel's tables: reactions grouped by kind, and per species the list of
    (reaction, net coefficient) that turns rates of progress into production rates."""
    import re
    from pelelm_gb300.mech.codegen import gen_tables
    from pelelm_gb300.workloads import load_mechanism
    for name in ("lidryer_syn", "drm19_syn", "gri_syn"):
        m = load_mechanism(name)
        txt = gen_tables(m, "global")

        def arr(nm):
            body = re.search(nm + r"\[[^\]]*\] = \{([^}]*)\}", txt).group(1)
            return [float(x.rstrip("ul")) if "." in x or "e" in x else int(x, 0) for x in body.split(",")]

        off, jj, nu = arr("kSpRxOff"), arr("kSpRxJ"), arr("kSpRxNu")
        # reaction order in the table: grouped by kind, stable within a kind
        kinds = {"elementary": 0, "three_body": 1, "falloff": 2}
        order = sorted(range(m.nr), key=lambda j: (kinds[m.reactions[j].kind], j))
        S = np.zeros((m.ns, m.nr))
        for jt, j in enumerate(order):
            r = m.reactions[j]
            for sp, v in r.products.items():
                S[m.index(sp), jt] += v
            for sp, v in r.reactants.items():
                S[m.index(sp), jt] -= v
        C = np.zeros_like(S)
        for k in range(m.ns):
            for e in range(off[k], off[k + 1]):
                C[k, jj[e]] += nu[e]
        assert np.array_equal(C, S), name
        # the lists are in reaction order (the gather sums in the order the per-thread RHS does)
        for k in range(m.ns):
            assert jj[off[k]:off[k + 1]] == sorted(jj[off[k]:off[k + 1]])


def test_gri_generator_species_saturated_and_recombinations_exothermic():
    from pelelm_gb300.mech.generate import _dH298
    from pelelm_gb300.mech.model import R_CAL
    from pelelm_gb300.workloads import load_mechanism
    m = load_mechanism("gri_syn")
    for s in m.species:
        c = s.composition
        assert c.get("H", 0) <= 2 * c.get("C", 0) + c.get("N", 0) + 2, s.name
    sp = {s.name: s for s in m.species}
    for r in m.reactions:
        if r.kind == "elementary":
            continue
        lhs = [n for n, v in r.reactants.items() for _ in range(v)]
        rhs = [n for n, v in r.products.items() for _ in range(v)]
        assert _dH298(sp, lhs, rhs) * R_CAL / 1000.0 < -20.0, r.equation()


def test_jacobian_program_replays_the_reaction_walk():
    """The cooperative setup's Jacobian contribution program (kJac* tables): replayed in numpy
    on random per-reaction partials it gives, entry for entry, the assembly by the reaction walk
    it replaces (each column k walks the reactions where k reacts or collides, in order, adding
    -+(W_i/W_k) v to every row slot i and -+W_i dq/dT to the T column of k); every nonzero entry
    is stored by exactly one lane, and the lanes' term streams (interleaved) are balanced."""
    import re
    from pelelm_gb300.mech.codegen import gen_tables
    from pelelm_gb300.workloads import load_mechanism
    rng = np.random.default_rng(4)
    for name in ("lidryer_syn", "drm19_syn", "gri_syn"):
        m = load_mechanism(name)
        txt = gen_tables(m, "global")

        def arr(nm, conv=int):
            body = re.search(nm + r"\[[^\]]*\] = \{([^}]*)\}", txt).group(1)
            return [conv(x.strip()) for x in body.split(",")]

        T = int(re.search(r"NJT = (\d+)", txt).group(1))
        codes = arr("kJacC", lambda x: int(x.rstrip("u")))
        negs = arr("kJacNeg", lambda x: int(x.rstrip("u")))
        effs = arr("kJacEffD", lambda x: float(eval(x)))
        ns, N = m.ns, m.ns + 1
        LDA = N + 1
        W = np.array([s.W for s in m.species])
        kinds = {"elementary": 0, "three_body": 1, "falloff": 2}
        order = sorted(range(m.nr), key=lambda j: (kinds[m.reactions[j].kind], j))
        idx = {s.name: i for i, s in enumerate(m.species)}
        P = rng.normal(size=(m.nr, 8)) * 10.0 ** rng.integers(-6, 6, size=(m.nr, 8))
        # the reaction walk, column by column
        A = np.zeros(N * LDA)
        for k in range(ns):
            for jt, j in enumerate(order):
                r = m.reactions[j]
                rs = [idx[s] for s, nu in r.reactants.items() for _ in range(nu)]
                ps = [idx[s] for s, nu in r.products.items() for _ in range(nu)]
                if not (k in rs or k in ps or r.kind != "elementary"):
                    continue
                v = 0.0
                for s_, sk in enumerate(rs):
                    if sk == k:
                        v += P[jt, 1 + s_]
                for s_, sk in enumerate(ps):
                    if sk == k:
                        v += P[jt, 4 + s_]
                if r.kind != "elementary":
                    v += P[jt, 7] * (1.0 + (r.efficiencies.get(m.species[k].name, 1.0) - 1.0))
                for row, i in enumerate(rs + ps):
                    sgn = -1.0 if row < len(rs) else 1.0
                    if i == k:
                        A[k * LDA + ns] += (sgn * W[i]) * P[jt, 0]
                    if v != 0.0:
                        A[i * LDA + k] += (sgn * (W[i] * (1.0 / W[k]))) * v
        # the program, lane by lane
        B = np.zeros(N * LDA)
        owner = {}
        terms = []
        for ln in range(32):
            acc, nterm, w = 0.0, 0, 0.0
            for t in range(T):
                c = 32 * t + ln
                code = codes[c]
                if code & (1 << 30):
                    i, k = divmod((code >> 9) & 0xFFF, LDA)
                    w = W[i] if k == ns else W[i] * (1.0 / W[k])
                pj = P[code & 0x1FF]
                if code & (1 << 21):
                    v = pj[0]
                else:
                    v = 0.0
                    for q in range(3):
                        if code & (1 << (22 + q)):
                            v += pj[1 + q]
                    for q in range(3):
                        if code & (1 << (25 + q)):
                            v += pj[4 + q]
                    if code & (1 << 28):
                        v += pj[7] * (effs[c] if code & (1 << 31) else 1.0)
                if (code & (1 << 21)) or v != 0.0:
                    acc += (-w if (negs[t] >> ln) & 1 else w) * v
                    nterm += 1
                if code & (1 << 29):
                    tg = (code >> 9) & 0xFFF
                    assert tg not in owner
                    owner[tg] = ln
                    B[tg] = acc
                    acc = 0.0
            terms.append(nterm)
        np.testing.assert_allclose(B, A, rtol=1e-12, atol=0)
        assert set(np.nonzero(A)[0].tolist()) <= set(owner), "a nonzero entry has no lane"
        assert max(terms) <= 1.5 * np.mean(terms) + 20, (name, terms)


def test_packed_reaction_records_match_the_reaction_table():
    """The warp and lane-group RHS read each reaction through two packed records (kRxArr,
    kRxPk); decoded, they must equal the fields of the FP64 reaction table entry by entry."""
    import re
    from pelelm_gb300.mech.codegen import gen_tables
    for name in ("lidryer_syn", "drm19_syn", "gri_syn"):
        txt = gen_tables(load_mechanism(name), "global")

        def rows(nm):
            body = re.search(nm + r"\[NR\] = \{\n(.*?)\n\};", txt, re.S).group(1)
            return [r.strip().rstrip(",") for r in body.split("\n")]

        def nums(row):
            return [float(x.rstrip("uf")) for x in re.findall(r"-?[0-9][0-9.e+-]*u?", row)]

        ref, arr, pk = rows("kReactionsD"), rows("kRxArr"), rows("kRxPk")
        assert len(ref) == len(arr) == len(pk) > 0
        for r, a, p in zip(ref, arr, pk):
            f = nums(r)  # lnA beta mEaR kind rev nr np rs0 rs1 rs2 ps0 ps1 ps2 dnu tb troe
            A = nums(a)
            x, y, z, w = (int(v) for v in nums(p))
            assert A[:3] == f[:3] and A[3] == 0.0 and w == 0
            kind, rev, nr, np_ = x & 3, (x >> 2) & 1, (x >> 3) & 3, (x >> 5) & 3
            dnu, tb, troe = ((x >> 7) & 15) - 8, ((x >> 11) & 2047) - 1, (x >> 22) - 1
            assert [kind, rev, nr, np_] == f[3:7]
            assert [dnu, tb, troe] == f[13:16]
            assert [(y >> (10 * s)) & 1023 for s in range(nr)] == f[7:7 + nr]
            assert [(z >> (10 * s)) & 1023 for s in range(np_)] == f[10:10 + np_]
