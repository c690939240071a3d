"""Q-atom connectivity (make_qconn, src/md.f90:9582-9620, with find_bonded's
recursive walk :9625-9680) and the Q-Q / Q-solute list nbqqlist
(:9716-9804), plus the skip data nbqplist reads (:10288, :10306).

The engine's start-up builds these on the host (qsource_gb300/system.py);
both the GPU kernels and the oracle's energies consume that one output.  Here
the oracle rebuilds them independently in C, literally as the reference does
(recursive depth-first walk, state by state), from the topology inputs the
start-up kept (solute bonds before shrink_topology, Q bonds, special
exclusions, soft pairs, Q-Q electrostatic scales), and every record must be
equal: same order, same LJ code, same scale, same skip flags and 1-4 pairs.
Systems: the reference's own test systems (sphere, periodic box, test2,
test3) and the synthetic ones with Q atoms inside a bonded solute."""
import numpy as np
import pytest

from conftest import golden_system


def _host_lists(s):
    per, k = [], 0
    nb = s.nbqq
    for st in range(int(s.nstates)):
        n = int(s.nbqq_count[st])
        per.append([(int(nb["iq"][k + r]), int(nb["j"][k + r]), int(nb["jq"][k + r]), int(nb["lj"][k + r]),
                     float(nb["els"][k + r])) for r in range(n)])
        k += n
    return per


def _check(s):
    from oracle.oracle import qconn_lists
    if not hasattr(s, "qconn_in"):
        pytest.skip("fixture written without the make_qconn inputs")
    qconn, per, skip, pairs = qconn_lists(s)
    nsol = int(s.nat_solute)
    assert per == _host_lists(s)
    assert np.array_equal(skip, np.asarray(s.qp_skip)[:nsol])
    host_pairs = [tuple(int(v) for v in r) for r in np.asarray(s.qp14_pairs).reshape(-1, 2)]
    assert pairs == host_pairs
    return qconn, per


@pytest.mark.parametrize("name", ["basic_sph", "basic_pbc", "test2", "test3"])
def test_reference_systems(name):
    _check(golden_system(name))


@pytest.mark.parametrize("cfg,kw", [(1, {}), (2, {}), (4, {}), (1, {"qvdw": True}), (2, {"vdw_rule": 2}),
                                    (5, {})])
def test_synthetic_systems(cfg, kw):
    from qsource_gb300 import synth
    s = synth.config(cfg, **kw)
    qconn, per = _check(s)
    # the solute systems put Q atoms inside a bonded chain: levels 2-4 occur
    if cfg in (2, 4, 5):
        assert {2, 3, 4} <= set(np.unique(qconn).tolist())
        assert any(r[3] == 3 for r in per[0])


def test_special_exclusion_and_qbond_change_the_lists():
    """A planted change in the inputs moves records: a special exclusion in
    state 1 only and a Q bond that exists in state 2 only."""
    from oracle.oracle import qconn_lists
    from qsource_gb300 import synth
    s = synth.config(2)
    base = qconn_lists(s)
    iq0, iq1 = int(s.iqseq[0]), int(s.iqseq[10])
    s.qconn_in = dict(s.qconn_in)
    s.qconn_in["exspec"] = np.array([[iq0, iq1, 1, 0]], np.int32)
    s.qconn_in["qbnd"] = np.array([[iq0, iq1, 0, 1]], np.int32)
    qconn, per, _, _ = qconn_lists(s)
    assert qconn[0, iq1, 0] == 0 and base[0][0, iq1, 0] == 9
    assert qconn[1, iq1, 0] == 2
    assert per != base[1]
