"""Writes tests/golden/*.json from the reference's own published result files.

Usage: python tests/golden/make_golden.py <path of a gogipav14/moljax checkout>.
The fixtures hold only the numbers the tests pin:
the FFT-CN error tables of benchmarks/results/precision_fp32_fp64.json and
benchmarks/results/scipy_comparison.json, the CN reactor conversions of
benchmarks/results/method_comparison_results.json, and the 3D FFT-CN errors and
times of benchmarks/results/3d_feasibility.json, the Gray-Scott method timings of
benchmarks/results/gray_scott.json, the penalty-RK4 reactor sweep of
benchmarks/results/reactor_results.json and the 1D solver comparison of
benchmarks/results/solver_comparison.json.
"""

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    res = os.path.join(ref, "benchmarks", "results")
    prec = json.load(open(os.path.join(res, "precision_fp32_fp64.json")))
    sc = json.load(open(os.path.join(res, "scipy_comparison.json")))
    out = {
        "source": "benchmarks/results/precision_fp32_fp64.json, scipy_comparison.json",
        "grid": 128, "L": 1.0,
        "precision_table": {
            "D": prec["config"]["D"], "t_final": prec["config"]["t_final"],
            "fp64": [{"dt": r["dt"], "n_steps": r["n_steps"], "error": r["error"]} for r in prec["fp64"]],
            "fp32": [{"dt": r["dt"], "n_steps": r["n_steps"], "error": r["error"]} for r in prec["fp32"]],
        },
        "scipy_comparison": {
            "D": sc["config"]["D"], "t_final": sc["config"]["t_final"],
            "n_steps": sc["config"]["fft_cn_steps"], "dt": sc["config"]["fft_cn_dt"],
            "numpy_error": sc["results"]["numpy_fft_cn"]["error"],
            "jax_error": sc["results"]["jax_fft_cn"]["error"],
        },
    }
    with open(os.path.join(HERE, "fftcn_published.json"), "w") as f:
        json.dump(out, f, indent=1)
    mc = json.load(open(os.path.join(res, "method_comparison_results.json")))
    reactor = {k: {"CN": {kk: v["CN"][kk] for kk in ("conversion", "steps", "dt", "t_final")},
                   "analytical": v.get("analytical")}
               for k, v in mc["reactor_methods"].items()}
    with open(os.path.join(HERE, "reactor_published.json"), "w") as f:
        json.dump({"source": "benchmarks/results/method_comparison_results.json",
                   "reactor_methods": reactor}, f, indent=1)
    f3 = json.load(open(os.path.join(res, "3d_feasibility.json")))
    with open(os.path.join(HERE, "fft3d_published.json"), "w") as f:
        json.dump({"source": "benchmarks/results/3d_feasibility.json", "config": f3["config"],
                   "experiments": [{k: e[k] for k in ("grid_size", "time_ms", "error")}
                                   for e in f3["experiments"] if e.get("success")]}, f, indent=1)

    rr = json.load(open(os.path.join(res, "reactor_results.json")))
    with open(os.path.join(HERE, "tubular_published.json"), "w") as f:
        json.dump({"source": "benchmarks/results/reactor_results.json", "N": 128, "t_final": 15.0,
                   "config": rr["config"],
                   "results": {k: {kk: v[kk] for kk in ("bc_type", "Pe", "Da", "conversion", "error", "dt",
                                                          "n_steps", "final_outlet_c", "mean_time")}
                               for k, v in rr["results"].items()}}, f, indent=1)
    gsb = json.load(open(os.path.join(res, "gray_scott.json")))
    with open(os.path.join(HERE, "gray_scott_published.json"), "w") as f:
        json.dump({"source": "benchmarks/results/gray_scott.json", "config": gsb["config"],
                   "methods": [{k: m_[k] for k in ("name", "time_s", "steps", "dt", "t_final")}
                               for m_ in gsb["methods"]]}, f, indent=1)
    so = json.load(open(os.path.join(res, "solver_comparison.json")))
    with open(os.path.join(HERE, "solver_comparison_published.json"), "w") as f:
        json.dump({"source": "benchmarks/results/solver_comparison.json", "config": so["config"],
                   "solvers": [{k: s_[k] for k in ("name", "steps", "dt", "rtol", "atol", "error_vs_scipy")
                                if k in s_} for s_ in so["solvers"]]}, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the gogipav14/moljax checkout>")
    main(sys.argv[1])
