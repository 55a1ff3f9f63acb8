"""The traversal's slab division (slab_div, aur_traverse.cuh) replaces the
IEEE division a / d by a reciprocal and one fused multiply-add correction
(Markstein's method) inside a checked range. Its results must equal the IEEE
quotient bit for bit there, or the node visits would differ from the
reference's slab test (ray.cuh:225-237). The checker is plain C with the C
library's correctly rounded fmaf, the same IEEE operations the GPU executes."""
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def test_slab_division_equals_ieee_division():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "slab_div_check")
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math",
                               os.path.join(HERE, "slab_div_check.c"), "-o", exe, "-lm"])
        out = subprocess.run([exe, "20000000"], capture_output=True, text=True)
    cases, accepted, bad = (int(x) for x in out.stdout.split())
    assert cases == 20000000 and accepted > 8000000
    assert bad == 0 and out.returncode == 0
