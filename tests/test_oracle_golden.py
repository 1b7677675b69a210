"""Pin the FP64 oracle against outputs of the reference's own CUDA kernels.

The fixtures in tests/golden were produced by tests/golden/make_golden.py on a
GB300 with the reference's gpuFunctionsImpl.cu compiled unmodified
(oracle/ref_harness).  Tolerances are those the oracle must meet to serve as
the parity checker: volume rel-L2 <= 2e-5 (parity bar 1e-4), k0 within
1e-4 px, modamps within 1e-5.
"""
import warnings

import numpy as np
import pytest

from golden_cases import CASES, DXY, load, rel_l2
from oracle.sirecon_oracle import SIMReconOracle, effective_nokz0, parse_config


def run_oracle(case):
    raw = case["raw"]
    o = SIMReconOracle(case["nx"], case["ny"], raw.shape[1], case["config"], case["otf"])
    o.ntimes = raw.shape[0]
    outs, k0s, amps = [], [], []
    for t in range(raw.shape[0]):
        o.set_raw(raw[t])
        o.load_and_rescale(t)
        o.set_cur_time(t)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            o.process()
        outs.append(o.result)
        k0s.append(o.k0.copy())
        amps.append(o.amp.copy())
    return np.stack(outs), np.stack(k0s), np.stack(amps)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    case, ref = load(name)
    out, k0, amp = run_oracle(case)
    if name == "c2d_128_q":
        # reference behaviour: the int-sized read of bNoKz0 excludes kz=0, and
        # in 2D that empties every overlap -> k0 = 0 and a NaN volume
        assert np.isnan(ref["result"]).all() or np.isnan(ref["result"]).any()
        assert np.isnan(out).any()
        assert np.all(ref["k0"] == 0) and np.all(k0 == 0)
        return
    dk = 1.0 / (case["nx"] * DXY)
    assert rel_l2(out, ref["result"]) < 2e-5
    assert np.abs(out - ref["result"]).max() / np.abs(ref["result"]).max() < 2e-5
    assert np.abs(k0 - ref["k0"]).max() / dk < 1e-4
    assert np.abs(amp - ref["amp"]).max() < 1e-5


@pytest.mark.parametrize("name", ["c3d_64", "c3d_96x80"])
def test_oracle_stages(name):
    case, ref = load(name)
    o = SIMReconOracle(case["nx"], case["ny"], case["raw"].shape[1], case["config"], case["otf"])
    o.set_raw(case["raw"][0])
    o.load_and_rescale(0)
    o.apodize()
    o.separate_bands()
    for b in range(5):
        assert rel_l2(o.bands[0][b], ref["sep_bands_dir0"][b]) < 1e-5
    # filter with the reference's own fit, on the reference's bands
    o.bands[0] = ref["sep_bands_dir0"].astype(np.complex128)
    o.k0 = ref["k0"][0].astype(np.float64)
    o.amp = ref["amp"][0].astype(np.complex128)
    o.filterbands(0)
    for b in range(5):
        assert rel_l2(o.bands[0][b], ref["filt_bands_dir0"][b]) < 1e-5


def test_effective_nokz0_rule():
    # wiener=0.001 -> 0x3A83126F: low half non-zero -> kz=0 excluded
    assert effective_nokz0(parse_config("wiener=0.001\n"))
    # wiener=2^-10 -> 0x3A800000: low half zero -> flag as declared
    assert not effective_nokz0(parse_config("wiener=0.0009765625\n"))
    assert effective_nokz0(parse_config("wiener=0.0009765625\nnokz0=1\n"))
    assert not effective_nokz0(parse_config("wiener=0.001\nreferenceFlagBytes=0\n"))
