"""Extract the reference's own golden test vectors into a small JSON fixture.

The reference project (Arcadia197/cmm-turbulence) pins its CUDA code with
golden monitoring files under Cuda-CMM/tests/*/data/reference-results_*/
Monitoring_data (raw little-endian float64 appended once per save instant,
written by src/ui/cmm-io.cu:508-534 and src/simulation/cmm-euler2d.cu:928-959).
This script copies the numbers (not any source code) for the Euler and
Vlasov-Poisson tests whose path is in scope, together with each test's input parameter file, into
tests/golden/reference_goldens.json so the tests never need the reference tree.

Usage:  python tests/golden/make_golden.py /path/to/reference
"""
import json
import os
import struct
import sys

TESTS = {
    # name: (results dir, input param file relative to Cuda-CMM/)
    "init_comp": ("tests/euler2D_init_fields/data/reference-results_comp_4_nodes_C256_F512_t1_T0",
                  "tests/euler2D_init_fields/params_comp.txt"),
    "init_conv": ("tests/euler2D_init_fields/data/reference-results_conv_4_nodes_C256_F512_t1_T0",
                  "tests/euler2D_init_fields/params_conv.txt"),
    "init_particles": ("tests/euler2D_init_fields/data/reference-results_particles_4_nodes_C256_F512_t1_T0",
                       "tests/euler2D_init_fields/params_particles.txt"),
    "init_zoom": ("tests/euler2D_init_fields/data/reference-results_zoom_4_nodes_C256_F512_t1_T0",
                  "tests/euler2D_init_fields/params_zoom.txt"),
    "init_forward": ("tests/euler2D_init_fields/data/reference-results_forward_4_nodes_C256_F512_t1_T0",
                     "tests/euler2D_init_fields/params_forward.txt"),
    "init_sample": ("tests/euler2D_init_fields/data/reference-results_sample_4_nodes_C256_F512_t1_T0",
                    "tests/euler2D_init_fields/params_sample.txt"),
    "one_step": ("tests/euler2D_one_step/data/reference-results_4_nodes_C256_F512_t1_T1",
                 "tests/euler2D_one_step/params.txt"),
    "remap_11b": ("tests/euler2D_11b_4nodes_reference_remapping/data/reference-results_4_nodes_C256_F512_t32_T2",
                  "examples/euler2D/params-11b-4nodes-reference-remapping.txt"),
    # restart: params-1 runs to t = 1 writing its MapStack, params-2 restarts from it to t = 2;
    # the goldens are those of the restarted run
    "restart_remap": ("tests/euler2D_remap/data/reference-results_4_nodes_C256_F512_t32_T2",
                      "tests/euler2D_remap/params-2.txt", "tests/euler2D_remap/params-1.txt"),
    "vlasov_15": ("tests/vlasov1D_15_vp_landau_damping/data/reference-results_C256_F512_t1024_T0.2",
                  "tests/vlasov1D_15_vp_landau_damping/params-15b-vp-landau-damping.txt"),
}


def read_f64(path):
    with open(path, "rb") as f:
        raw = f.read()
    n = len(raw) // 8
    return list(struct.unpack("<%dd" % n, raw[: 8 * n]))


def main(ref_root):
    base = os.path.join(ref_root, "Cuda-CMM")
    out = {}
    for name, (res_dir, param_file, *pre) in TESTS.items():
        rdir = os.path.join(base, res_dir, "Monitoring_data")
        entry = {"params_in": open(os.path.join(base, param_file)).read(), "files": {}}
        if pre:
            entry["params_pre"] = open(os.path.join(base, pre[0])).read()
        for root, _, files in os.walk(rdir):
            for fn in sorted(files):
                if not fn.endswith(".data") or fn.endswith("_Hash.data") or fn == "Time_c.data":
                    continue
                rel = os.path.relpath(os.path.join(root, fn), rdir)[: -len(".data")]
                entry["files"][rel] = read_f64(os.path.join(root, fn))
        out[name] = entry
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print("wrote", dst, sum(len(v["files"]) for v in out.values()), "series")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
