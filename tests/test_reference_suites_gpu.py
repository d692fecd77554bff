"""The reference's own unit-test suites, compiled unchanged against the GPU
drop-in accelerator (skwarka_gb300/adapter: the reference's
TriangleAccelerator class over the C ABI, replacing the reference's
TriangleAccelerator.h / .cpp in its build) and run on the GPU.

* TriangleAccelerator.test.h: world bounds, closest hits against brute
  force (t within 1e-9), the "no self re-hit" epsilon test (1000 x 1000
  outgoing rays with GetNextMinT), any hit against brute force, and the
  10,000-tetrahedra instancing test;
* Scene.test.h: Scene::Intersect / IntersectTest over the drop-in (the
  reference's Scene holds the accelerator by value, Scene.h:99);
* LTEIntegrator.test.h: the integrator's radiance through Scene::Intersect.

Every suite must report CxxTest's "OK!"."""
import subprocess

import pytest

import reference_suites

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("suite", ["TriangleAccelerator", "Scene", "LTEIntegrator"])
def test_reference_suite_on_gpu(gpu, suite):
    if not reference_suites.available():
        pytest.skip("the reference's staged sources and CxxTest are not on this machine")
    exe = reference_suites.build_runner([suite])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    print(f"[{suite} suite on the GPU drop-in]\n{r.stdout[-2000:]}{r.stderr[-2000:]}")
    assert r.returncode == 0 and "OK!" in r.stdout
