"""Times the reference's own CPU implementation, Code/test/test_timesC.py
(`kshape(x, k)`, test_timesC.py:267-276 and :213-264), on the host cores.

Runs only where the reference tree is present (TIMESC_REFERENCE, else the
directory `reference` beside the repository): the Python reference does not
reach GPU hosts.  numpy >= 2 removed np.Inf, which the file uses; the alias is
restored before import.  np.random is seeded (its initial labels are the
first randint draw, test_timesC.py:217), BLAS threads are the host's cores, and
its per-iteration prints are swallowed.  The series are the engine's synthetic
workloads from the oracle library's copy of the generator.

    python oracle/time_pyref.py [c1] [c2s]

c1:  n=300, m=128, k=4 (the labelled CPU-sized configuration);
c2s: n=2000, m=2709, k=8 - a tenth of the n=20,000 configuration, whose
     n x k x 8192 complex128 temporaries (21 GB each) do not fit the host.
Prints one JSON line per case: seconds per call, iterations, pairs/s.
"""
import contextlib
import importlib.util
import io
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = os.environ.get("TIMESC_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))

CASES = {
    "c1": (300, 128, 4, 0.2, 0.0),
    "c2s": (2000, 2709, 8, 0.2, 2.0),
}


def main():
    cores = str(len(os.sched_getaffinity(0)))
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ.setdefault(v, cores)
    import numpy as np
    if not hasattr(np, "Inf"):
        np.Inf = np.inf
    path = os.path.join(REF, "Code", "test", "test_timesC.py")
    if not os.path.exists(path):
        raise SystemExit("the reference's test_timesC.py is not present here")
    spec = importlib.util.spec_from_file_location("test_timesC", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    for name in (sys.argv[1:] or ["c1"]):
        n, m, k, noise, dirichlet = CASES[name]
        data, _ = O.generate(n, m, k, noise=noise, dirichlet=dirichlet, seed=0)
        x = data.astype(np.float64)
        reps = 3 if n * m <= 1e6 else 1
        times, iters = [], []
        # every iteration computes its distances with one _ncc_c_3dim call (test_timesC.py:255);
        # the iteration count it returns reuses a loop variable of the inner loops (:226-241)
        ncc3, calls = mod._ncc_c_3dim, [0]

        def counted(*a):
            calls[0] += 1
            return ncc3(*a)

        mod._ncc_c_3dim = counted
        for r in range(reps):
            np.random.seed(r)
            calls[0] = 0
            t0 = time.perf_counter()
            with contextlib.redirect_stdout(io.StringIO()):
                mod.kshape(x, k)
            times.append(time.perf_counter() - t0)
            iters.append(calls[0])
        mod._ncc_c_3dim = ncc3
        t = min(times)
        n_it = iters[times.index(t)]
        print(json.dumps({"case": name, "n": n, "m": m, "k": k, "cores": int(cores), "seconds": t,
                          "iterations": n_it, "seconds_per_iteration": t / n_it,
                          "pairs_per_s": n * k * n_it / t, "all_seconds": times}))


if __name__ == "__main__":
    main()
