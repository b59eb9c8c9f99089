"""Pins the tracking file that the engine's local driver writes (`--tracking --out`) to the reference's
own reader, experiments/show.py.

Two steps, on two machines:

    python tests/golden/make_tracking_golden.py write OUT.bin     # where a GPU is: run the driver
    python tests/golden/make_tracking_golden.py parse OUT.bin     # here: REF_ROOT=<reference tree>

`write` runs one bin_fednl_local command line through doptExecuteLocal (the problem of
tests/test_local_driver.py, TopK, 12 rounds) and copies the tracking file to OUT.bin.  `parse` runs the
reference's show.py on that file unchanged (its plotting library replaced by a recording stub: only the
parser's results are wanted) and writes tests/golden/tracking_show.npz: the file's bytes and every header
field and per-round series show.py read from them.  tests/test_local_driver.py then checks the engine's
own reading of the committed bytes against show.py's, and a fresh run's file against the same layout.
"""
import os
import runpy
import shutil
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
COMMAND = ("--train_dataset {data} --clients 6 --reshuffle_train --add_intercept --lambda 0.001 --rounds 12 "
           "--workers 3 --algorithm fednl1 --compressor topk --k_compressor_as_d_mult 2 --fednl-option-b "
           "--tracking --out {out} --debug forcesequpdate --use_theoretical_alpha_option_2 --theoretical_alpha")


def write_libsvm(path, prob):
    with open(path, "w") as f:
        for s in range(prob.total_samples):
            a = prob.features[s]
            items = " ".join(f"{i + 1}:{int(a[i])}" for i in range(prob.d) if a[i] != 0.0)
            f.write(f"{'+1' if prob.labels[s] > 0 else '-1'} {items}\n")


def tracking_problem():
    from ufednl_gb300 import datagen
    prob = datagen.binary_problem(41, 16, [30] * 6, 0.3, 1e-3)       # last attribute = intercept
    return datagen.Problem(prob.d - 1, prob.n_samples, prob.features[:, :-1], prob.labels, prob.lam)


def write(out_bin):
    from ufednl_gb300 import build, fednl
    build.build()
    tmp = tempfile.mkdtemp()
    data = os.path.join(tmp, "data.txt")
    write_libsvm(data, tracking_problem())
    out = os.path.join(tmp, "track_{algorithm}_{dataset}.bin")
    rc, _ = fednl.execute_local(COMMAND.format(data=data, out=out))
    if rc != 0:
        raise SystemExit(f"the driver returned {rc}")
    shutil.copyfile(os.path.join(tmp, "track_fednl1_data.bin"), out_bin)


class _Recorder(types.ModuleType):
    """Stands in for the plotting modules: every attribute is a callable that returns another one."""

    def __getattr__(self, name):
        return _Recorder(name)

    def __call__(self, *a, **k):
        return _Recorder("call")

    def __getitem__(self, i):
        return _Recorder("item")

    def __setitem__(self, i, v):
        pass

    def __iter__(self):
        return iter(())


def parse(in_bin):
    ref = os.environ.get("REF_ROOT")
    if not ref:
        raise SystemExit("set REF_ROOT to the reference tree")
    show = os.path.join(ref, "experiments", "show.py")
    stub = _Recorder("matplotlib")
    saved = {k: sys.modules.get(k) for k in ("matplotlib", "matplotlib.pyplot", "matplotlib.ticker")}
    sys.modules.update({"matplotlib": stub, "matplotlib.pyplot": stub, "matplotlib.ticker": stub})
    argv = sys.argv
    sys.argv = [show, in_bin]
    try:
        g = runpy.run_path(show, run_name="__main__")
    finally:
        sys.argv = argv
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    raw = np.frombuffer(open(in_bin, "rb").read(), dtype=np.uint8)
    fields = dict(
        raw=raw,
        dataset=np.array(g["dataset"]), algorithm=np.array(g["algorithm"]), compressor=np.array(g["compressor"]),
        ints=np.array([g["totalSamplesPerClient"], g["totalSamples"], g["roundsTotal"], g["nClients"], g["d"],
                       g["k_for_fednl_c_abs"]], dtype=np.int64),
        doubles=np.array([g["k_for_fednl_c_mult_d"], g["global_lr"], g["alpha_lr"], g["lambda_regul"]]),
        rounds=np.array(g["rounds"], dtype=np.int64), grad_norm=np.array(g["gradsNorm"]),
        func_value=np.array(g["funcValue"]), x_norm=np.array(g["xiNorm"]),
        send_bits_total=np.array(g["sendBitsTotal"]), send_bits_indices=np.array(g["sendBitsIndicies"]),
        elapsed=np.array(g["eclapsedTime"]))
    np.savez(os.path.join(HERE, "tracking_show.npz"), **fields)
    print("rounds", len(fields["rounds"]), "header", fields["ints"], fields["doubles"])


if __name__ == "__main__":
    if len(sys.argv) != 3 or sys.argv[1] not in ("write", "parse"):
        raise SystemExit(__doc__)
    (write if sys.argv[1] == "write" else parse)(sys.argv[2])
