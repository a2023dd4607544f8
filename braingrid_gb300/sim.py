"""A BrainGrid run from its parameter files on the GPU: the reference's growth driver
(Core/BGDriver.cpp, Core/Simulator.cpp:140-190) with this library as the model.

    python -m braingrid_gb300.sim -t config.xml [-s stim.xml] [-o result.xml] [-r state] [-w state]
                                  [-d device] [--noise device]

reads the parameter file (braingrid_gb300.config), sets the network up as the reference does,
runs numSims epochs of Tsim seconds with the epoch pass at each end (ConnGrowth's growth and
recorder, or the plain recorder), and writes the reference's result file (braingrid_gb300.
results) to -o, or to the file's stateOutputFileName; -r and -w read and write the reference's
checkpoint stream as the driver's flags of those names do.  With the reference's noise stream (the
default) the result file is the reference's, byte for byte, wherever the run is bit-exact (see
the parity tests): the noise and a Poisson stimulus's intervals are the reference's own draws,
made on the host.  --noise device draws both on the GPU instead.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import config as cf
from . import lib as bg
from . import results


IF_SETUP = ("Cm", "Rm", "Vrest", "Vinit", "Iinject", "Tau")


def simulate(p, noise="reference", arrays=None, restore=None, save=False,
             max_chunk_values=1 << 24):
    """Runs p (config.Params); returns dict(text=result file, seconds=wall time of the epochs,
    steps=simulation steps, error_word=the device error word, stream=the reference's checkpoint
    stream at the end when save).  restore: a checkpoint stream loaded after setup, as the
    reference driver's -r does (Core/BGDriver.cpp:88-94: the model's state, then the recorder's
    start values; the run then starts at step 0)."""
    a = arrays if arrays is not None else cf.setup(p)
    inject = noise == "reference"
    net = cf.network(p, a, noise_mode=bg.BG3_NOISE_INJECT if inject else bg.BG3_NOISE_DEVICE)
    try:
        N, spe = a["N"], p.steps_per_epoch
        growth_conn = p.conn_class == "ConnGrowth"
        if_fields = {k: a[k] for k in IF_SETUP}
        if restore is not None:
            extra = net.deserialize(restore, growth=growth_conn, step=0)
            if_fields = {k: extra[k] for k in IF_SETUP}
        gen = bg.NormStream(p.seed) if inject else None
        if inject and "poisson" in a:
            # the reference's own intervals, drawn ahead on its global generator
            net.push_poisson_isis(*cf.poisson_intervals(a, spe * p.epochs + 1))
        chunk = max(1, min(spe, max_chunk_values // max(N, 1)))
        growth = p.conn_class == "ConnGrowth"
        t0 = time.perf_counter()
        # the next chunk's noise is drawn on the host while the GPU runs the current chunk (the
        # steps are queued asynchronously; the push waits for them); at most one value per
        # neuron per step is consumed and what is left over stays queued for the next chunk
        pending = gen.take(N * chunk) if inject else None
        for e in range(p.epochs):
            done = 0
            while done < spe:
                k = min(chunk, spe - done)
                if inject:
                    net.push_noise(pending)
                net.step(k)
                if inject:
                    pending = gen.take(N * chunk)
                done += k
            if growth:
                net.growth(e + 1)
            else:
                net.record()
        net.sync()
        seconds = time.perf_counter() - t0
        err = net.error_word
        vthresh = net.download_lif(fields=("Vthresh",))["Vthresh"]
        text = results.state_xml(growth, N, p.epochs, p.tsim, cf.DELTA_T, net.sim_step,
                                 net.download_histories(), a["xloc"], a["yloc"], a["ntype"],
                                 a["starter"], vthresh)
        if gen is not None:
            gen.close()
        stream = net.serialize(growth=growth_conn, **if_fields) if save else None
        return dict(text=text, seconds=seconds, steps=net.sim_step, error_word=err, stream=stream)
    finally:
        net.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("-t", "--config", required=True, help="parameter file")
    ap.add_argument("-s", "--stim", default=None, help="stimulus file")
    ap.add_argument("-o", "--output", default=None, help="result file (default: the "
                    "parameter file's stateOutputFileName)")
    ap.add_argument("-r", "--read-state", default=None,
                    help="checkpoint stream to start from (the reference driver's -r)")
    ap.add_argument("-w", "--write-state", default=None,
                    help="write the checkpoint stream at the end (the reference driver's -w)")
    ap.add_argument("-d", "--deviceid", type=int, default=None, help="CUDA device id")
    ap.add_argument("--noise", choices=("reference", "device"), default="reference")
    a = ap.parse_args(argv)
    if a.deviceid is not None:
        bg.set_device(a.deviceid)
    p = cf.read(a.config, a.stim)
    restore = None
    if a.read_state:
        with open(a.read_state, "rb") as f:
            restore = f.read()
    r = simulate(p, a.noise, restore=restore, save=bool(a.write_state))
    if a.write_state:
        with open(a.write_state, "wb") as f:
            f.write(r["stream"])
    out = a.output or p.output
    if out:
        d = os.path.dirname(out)
        if d:
            os.makedirs(d, exist_ok=True)
        with open(out, "w") as f:
            f.write(r["text"])
    sim_s = float(np.float32(p.tsim) * np.float32(p.epochs))
    print(json.dumps({"output": out, "simulated_s": sim_s, "wall_s": round(r["seconds"], 3),
                      "steps": r["steps"], "error_word": r["error_word"]}))
    return 0 if r["error_word"] == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
