"""Parity at the benchmark's full sizes, through properties that do not depend on size.

  - Widom, 20,000 CO2 insertions into the 3,456-atom silica (the Widom workload): mixed and
    FP64 select the same trials for at least 99.9 % of the insertions, and a spread
    sample of insertions recomputed alone by the FP64 oracle (same Philox counters) match
    the GPU's FP64 results exactly (selections, Rosenbluth weights to 1e-10) and its mixed
    results to 2e-6.
  - GCMC, 456 chains (three per SM, replicas of one framework) for 200 steps: at least 95 %
    of the chains take the same decisions in mixed as in FP64, and sampled chains take the
    FP64 oracle's decisions exactly. Every chain whose mixed and FP64 runs part is replayed
    step by step to its first divergent step; the FP64 oracle, continuing the same chain,
    shows that step's closest decision (a trial selection or an acceptance) within 1e-6 of
    a tie in relative weight (about beta |dE|): the runs part only where a 1e-6 perturbation
    may flip a decision.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import co2_system
from tests.test_gpu_gcmc import ora_params
from tests.test_gpu_parity import _fields, oracle_widom

pytestmark = pytest.mark.gpu


def test_widom_full_size(grx_lib):
    s = co2_system(n_co2=0)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 16])
    box.ewald_total()
    d = grx_lib.widom_desc(s, 1, 10, 10, seed=42)
    n = 20000
    g64 = box.widom(d, 0, n, prec=grx_lib.GRX_FP64)
    gm = box.widom(d, 0, n, prec=grx_lib.GRX_MIXED)
    box.close()
    same = (g64["sel_first"] == gm["sel_first"]) & (g64["sel_orient"] == gm["sel_orient"])
    assert same.mean() >= 0.999
    for i in (0, 1, 137, 2500, 9999, 14001, 19998, 19999):
        ref, _ = oracle_widom(s, 1, 1, first_move=i)
        R, sf, so, ok, _ = _fields(ref)
        assert g64["sel_first"][i] == sf[0] and g64["sel_orient"][i] == so[0]
        assert abs(g64["rosenbluth"][i] - R[0]) <= 1e-10 * max(R[0], 1e-300)
        if R[0] > 0 and gm["sel_first"][i] == sf[0] and gm["sel_orient"][i] == so[0]:
            assert abs(gm["rosenbluth"][i] - R[0]) <= 2e-6 * R[0]


def test_gcmc_full_size_chains(grx_lib):
    s = co2_system(n_co2=0)
    nfw = s["comp_start"][1]
    R = 456
    descs = [grx_lib.gcmc_desc(1, ntrials=10, norient=10, p_translation=0.25, p_rotation=0.5, p_reinsertion=0.5,
                               p_swap=1.0, pressure_pa=1e5, seed=42, stream=k) for k in range(R)]
    res = {}
    for name, p in (("fp64", grx_lib.GRX_FP64), ("mixed", grx_lib.GRX_MIXED)):
        parent = grx_lib.Box(s, capacity=[nfw, 3 * 160])
        parent.ewald_total()
        boxes = [parent] + [parent.replica() for _ in range(R - 1)]
        res[name] = grx_lib.gcmc_run(boxes, descs, 0, 200, p)
        for b in reversed(boxes):
            b.close()
    same = [list(a.accepted) == list(b.accepted) and a.n_molecules == b.n_molecules
            for a, b in zip(res["fp64"], res["mixed"])]
    assert np.mean(same) >= 0.95
    S = O.OracleSystem(s)
    for k in (0, 211, 455):
        ost, _, _ = S.gcmc(ora_params(descs[k]), [nfw, 3 * 160], 0, 200)
        assert list(res["fp64"][k].accepted) == list(ost.accepted)
        assert res["fp64"][k].n_molecules == ost.n_molecules
    # the divergent chains: first divergent step, and the oracle's decision margin there
    div = [k for k in range(R) if not same[k]]
    if not div:
        return
    runs = {}
    for name, p in (("fp64", grx_lib.GRX_FP64), ("mixed", grx_lib.GRX_MIXED)):
        parent = grx_lib.Box(s, capacity=[nfw, 3 * 160])
        parent.ewald_total()
        runs[name] = [parent] + [parent.replica() for _ in range(len(div) - 1)]
    sub = [descs[k] for k in div]
    first_div = {}
    acc = {n: [np.zeros(5, dtype=np.int64) for _ in div] for n in runs}
    for step in range(200):
        st = {n: grx_lib.gcmc_run(runs[n], sub, step, 1, p)
              for n, p in (("fp64", grx_lib.GRX_FP64), ("mixed", grx_lib.GRX_MIXED))}
        for j, k in enumerate(div):
            if k in first_div:
                continue
            for n in runs:
                acc[n][j] += np.array(st[n][j].accepted)
            nf, nm = st["fp64"][j].n_molecules, st["mixed"][j].n_molecules
            diff = not np.array_equal(acc["fp64"][j], acc["mixed"][j]) or nf != nm
            if not diff and nf > 0:
                pf = runs["fp64"][j].positions(1, 3 * nf)
                pm = runs["mixed"][j].positions(1, 3 * nm)
                diff = np.max(np.abs(pf - pm)) > 1e-6
            if diff:
                first_div[k] = step
        if len(first_div) == len(div):
            break
    for n in runs:
        for b in reversed(runs[n]):
            b.close()
    report = []
    for k in div:
        step = first_div[k]
        ch = O.OracleChain(S, ora_params(descs[k]), [nfw, 3 * 160])
        if step > 0:
            ch.run(0, step)
        last = ch.run(step, 1)[0]
        report.append((k, step, last.last_margin))
    print("divergent chains (chain, first divergent step, oracle decision margin):", report)
    assert all(m <= 1e-6 for _, _, m in report), report
