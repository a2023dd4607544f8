"""Pins the oracle's checkpoint stream (bgo_serialize) to the reference's: the bytes
Simulator::serialize wrote at the end of each case's run (tests/golden/serialize.npz, made by
tests/golden/make_golden.py with the compiled reference) are reproduced byte for byte."""
import numpy as np
import pytest

from tests.golden.configs import case
from tests.netcases import oracle_from_case, steps_per_epoch

SER_CASES = ["c0_grown", "c0_spiking", "c0_stdp", "izh_dstdp", "izh_static", "ragged", "ragged_izh"]


def run_to_end(name):
    c = case(name)
    o = oracle_from_case(c)
    spe = steps_per_epoch(c)
    for e in range(c["epochs"]):
        o.step_n(spe)
        if c.get("static"):
            o.record_static()
        else:
            o.growth()
            o.record_epoch(e + 1)
    return c, o


def tokens(b):
    return bytes(b).split(b"\0")


def comparable(b, c):
    """The stream's tokens with each neuron's Isyn masked: the reference allocates Isyn and never
    sets it (Neurons/AllIFNeurons.cpp:46), so its stream carries whatever the heap held there
    (zeros in most runs, other values in some); every other byte is compared."""
    t = tokens(b)
    per = 23 if c.get("neuron") == "izh" else 17
    for i in range(c["N"]):
        t[1 + i * per + 9] = b"<Isyn>"
    return t


@pytest.mark.parametrize("name", SER_CASES)
def test_oracle_stream_matches_reference(name):
    c, o = run_to_end(name)
    want = np.load("tests/golden/serialize.npz")[name].tobytes()
    got = o.serialize(conn_growth=not c.get("static"))
    tg, tw = comparable(got, c), comparable(want, c)
    if tg != tw:
        bad = [i for i, (a, b) in enumerate(zip(tg, tw)) if a != b]
        raise AssertionError("%s: %d vs %d tokens, first differences %r" % (
            name, len(tg), len(tw), [(i, tg[i], tw[i]) for i in bad[:5]]))
    # the stream carries the whole synapse population the reference had
    assert int(tokens(want)[1 + c["N"] * (23 if c.get("neuron") == "izh" else 17)]) == o.total
