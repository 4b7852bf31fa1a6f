"""The device collision routines, compiled for the host, against the oracle.

ak_lattice.cuh's collide (deviation form, used for FP32 arithmetic) and
collide_full (the FP64 kernel's form, also evaluated in double-float
arithmetic for the df64 form) are __host__ __device__; this test
builds a small host program with nvcc that runs both on random cells and
compares them with the oracle's cumulant collision (no GPU needed).
"""
import os
import subprocess
import tempfile
from pathlib import Path

import pytest

from aerokinetic_gb300 import _native

O = pytest.importorskip("oracle.oracle")

PROGRAM = r'''
#include <cstdio>
#include <cmath>
#include <random>
#include "ak_lattice.cuh"
#include <cstdlib>
extern "C" void ako_collide_cells_sgs(double *g, long long n, double ws, double wb, double c18);
int main(int argc, char **argv) {
    const double C = argc > 1 ? atof(argv[1]) : 0.0, c18 = 18.0 * C * C;
    std::mt19937_64 rng(5);
    std::normal_distribution<double> N(0, 1);
    double worst_full = 0, worst_dev = 0, worst_f32 = 0, worst_df = 0;
    for (int t = 0; t < 2000; ++t) {
        double rho = 1 + 0.05 * N(rng), u[3] = {0.08 * N(rng), 0.08 * N(rng), 0.08 * N(rng)};
        double g[27], a[27], b[27], c[27];
        float f[27];
        ak::df64 h[27];
        for (int q = 0; q < 27; ++q) {
            double p = rho;
            int e[3] = {ak::cx(q), ak::cy(q), ak::cz(q)};
            for (int k = 0; k < 3; ++k) p *= e[k] == 0 ? 2.0/3 - u[k]*u[k] : 0.5*(1.0/3 + u[k]*u[k] + e[k]*u[k]);
            g[q] = p - ak::weight(q) + 3e-3 * N(rng) * ak::weight(q);
            a[q] = b[q] = c[q] = g[q];
            f[q] = (float)g[q];
            h[q] = ak::df64(g[q]);
        }
        double ws = 1.0 + 0.999 * (t % 100) / 100.0, wb = (t % 3 == 0) ? 1.0 : 0.7;
        ak::Sgs<double> md;
        ak::Sgs<float> mf;
        ak::Sgs<ak::df64> mh;
        if (c18 > 0) {
            md.tau0 = mh.tau0 = 1.0 / ws;
            md.c18 = mh.c18 = c18;
            mf.tau0 = (float)(1.0 / ws);
            mf.c18 = (float)c18;
        }
        ak::collide_full<double>(a, 1.0 - ws, wb, md);
        ak::collide<double>(b, ws, wb, md);
        ak::collide<float>(f, (float)ws, (float)wb, mf);
        ak::collide_full<ak::df64>(h, ak::df64(1.0 - ws), ak::df64(wb), mh);
        ako_collide_cells_sgs(c, 1, ws, wb, c18);
        for (int q = 0; q < 27; ++q) {
            worst_full = fmax(worst_full, fabs(a[q] - c[q]));
            worst_dev = fmax(worst_dev, fabs(b[q] - c[q]));
            worst_f32 = fmax(worst_f32, fabs((double)f[q] - c[q]));
            worst_df = fmax(worst_df, fabs((double)h[q] - c[q]));
        }
    }
    printf("%.6e %.6e %.6e %.6e\n", worst_full, worst_dev, worst_f32, worst_df);
    return 0;
}
'''


@pytest.mark.parametrize("smagorinsky", [0.0, 0.1, 0.25])
def test_device_collision_forms_match_oracle_on_host(smagorinsky):
    """Molecular viscosity and the Smagorinsky shear rate (C = 0.1, 0.25)."""
    nvcc = _native.nvcc()
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        (tmp / "main.cu").write_text(PROGRAM)
        obj = tmp / "oracle.o"
        subprocess.run(["gcc", "-O2", "-fopenmp", "-c", "-o", str(obj), str(O.SOURCE)], check=True)
        exe = tmp / "check"
        subprocess.run([nvcc, "-std=c++17", "-O2", "-I", str(_native.PACKAGE / "csrc"), "-o", str(exe),
                        str(tmp / "main.cu"), str(obj), "-Xcompiler", "-fopenmp", "-lgomp", "-lm"],
                       check=True, capture_output=True)
        out = subprocess.run([str(exe), repr(smagorinsky)], check=True, capture_output=True, text=True).stdout.split()
    full, dev, f32, df = map(float, out)
    assert full < 2e-15 and dev < 2e-15
    assert f32 < 2e-6
    # double-float (48-bit) arithmetic: far inside the 2e-12 per-population bar
    assert df < 5e-14
