"""qgpu_lrf_scan_static, the scan entry point that allocates no device memory.

It serves callers that may not call cudaMalloc -- a program whose device
memory belongs to its own allocator or to a pool reserved once at start-up,
or a time-step loop where an allocation (which can synchronise the device) is
not allowed.  Such a caller passes every input and output buffer itself (here
torch allocates them, standing in for the caller's allocator); the entry point
keeps its partial sums in a fixed array of the library.

Its results are checked against the engine's own list build (qgpu_build_lists
with qgpu_get_lrf and qgpu_get_group_pairs) with the tolerances of the LRF
parity test: group centres to 1e-12, each multipole family to 1e-5 of its
largest entry, near-group counts exactly.  Two calls in a row on systems of
different sizes show that the shared array's leftover contents do not leak
into the next call.  The file name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

LRF_FAMILIES = ((3, 4), (4, 7), (7, 16), (16, 43))   # phi0, phi1, phi2, phi3


def _device_inputs(s):
    """The caller-side device arrays of one system (charge groups in topology
    order, Q-atom charges zeroed so they do not feed the multipoles)."""
    import torch
    dev = torch.device("cuda:0")
    ngroup = len(s.cgp_first)
    crg = np.array(s.crg, dtype=np.float64)
    crg[np.asarray(s.iqatom) >= 0] = 0.0
    members = [np.asarray(s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]) for g in range(ngroup)]
    g_start = np.zeros(ngroup + 1, dtype=np.int32)
    g_start[1:] = np.cumsum([len(m) for m in members])
    g_atoms = np.concatenate(members).astype(np.int32)
    g_switch = np.asarray(s.cgp_switch, dtype=np.int32)
    g_flags = (np.arange(ngroup) >= s.ncgp_solute).astype(np.int32)
    g_flags |= 2 * np.asarray(s.excl)[g_switch].astype(np.int32)

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    return {"ngroup": ngroup, "x": t(np.asarray(s.x, dtype=np.float64)), "crg": t(crg), "g_start": t(g_start),
            "g_atoms": t(g_atoms), "g_switch": t(g_switch), "g_flags": t(g_flags),
            "lrf43": torch.full((ngroup, 43), np.nan, dtype=torch.float64, device=dev),
            "near": torch.full((ngroup,), -1, dtype=torch.int32, device=dev)}


def _scan_static(lib, s, d):
    import torch
    p = lambda a: C.c_void_p(a.data_ptr())
    origin = (C.c_double * 3)(*[float(v) for v in s.xwcent])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.qgpu_lrf_scan_static(d["ngroup"], p(d["x"]), p(d["crg"]), p(d["g_start"]), p(d["g_atoms"]),
                                  p(d["g_switch"]), p(d["g_flags"]), origin, s.Rcpp, s.Rcpw, s.Rcww, s.RcLRF,
                                  p(d["lrf43"]), p(d["near"]), stream)
    torch.cuda.synchronize()
    from qsource_gb300.abi import last_error
    assert rc == 0, last_error(lib)
    return d["lrf43"].cpu().numpy(), d["near"].cpu().numpy()


def _engine_reference(s):
    from qsource_gb300.engine import Engine
    e = Engine(s)
    e.make_pair_lists()
    lrf = e.lrf(0)
    pairs = e.group_pairs(0)
    near = np.bincount(pairs.ravel(), minlength=len(s.cgp_first)) if len(pairs) else np.zeros(len(s.cgp_first))
    e.close()
    return lrf, near


def _check(got_lrf, got_near, ref_lrf, ref_near):
    assert np.all(np.isfinite(got_lrf))
    assert np.allclose(got_lrf[:, :3], ref_lrf[:, :3], rtol=0, atol=1e-12)
    for lo, hi in LRF_FAMILIES:
        scale = np.abs(ref_lrf[:, lo:hi]).max()
        err = np.abs(got_lrf[:, lo:hi] - ref_lrf[:, lo:hi]).max()
        assert err <= 1e-5 * scale, (lo, err, scale)
    assert np.array_equal(got_near, ref_near)


@pytest.mark.gpu
def test_static_scan_matches_engine_on_two_calls(engine_lib):
    from qsource_gb300 import synth
    # the scan applies the switch-atom cut-off (iuse_switch_atom = 1)
    big, small = synth.config(2, any_atom=False), synth.config(1)
    assert big.use_LRF and small.use_LRF
    assert len(big.cgp_first) > len(small.cgp_first)
    first = _scan_static(engine_lib, big, _device_inputs(big))
    second = _scan_static(engine_lib, small, _device_inputs(small))
    _check(*first, *_engine_reference(big))
    _check(*second, *_engine_reference(small))


def test_static_scan_refuses_oversize_input(engine_lib):
    """More groups than the fixed scratch holds: refused before any device work."""
    from qsource_gb300.abi import last_error
    dummy = C.c_void_p(16)
    origin = (C.c_double * 3)(0.0, 0.0, 0.0)
    rc = engine_lib.qgpu_lrf_scan_static(65537, dummy, dummy, dummy, dummy, dummy, dummy, origin, 10.0, 10.0,
                                         10.0, 99.0, dummy, dummy, None)
    assert rc == 1
    assert "65536" in last_error(engine_lib)
