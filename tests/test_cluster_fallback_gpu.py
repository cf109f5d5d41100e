"""The one-CTA forms of the cluster kernels (extrusion of several layers, blocked DM transpose, EFC step), which run
where thread-block clusters cannot be launched, against the cluster forms: HX_NO_CLUSTERS=1 selects them in a
child process, which writes its results for the same seeded inputs; the parent computes them with clusters.
Tolerances: the two forms add the same terms in different groupings (float64 1e-13, float32 1e-6 relative)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')

_CHILD = r'''
import sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[2])
import hcipy_gb300 as hg
from hcipy_gb300.kernels import SparseBasis
import scipy.sparse as sp

out = {}
# three float32 layers evolved as one batch, and a float64 pair
for name, dtype, n in (('atm32', torch.float32, 48), ('atm64', torch.float64, 40)):
    grid = hg.make_pupil_grid(n, 2.0)
    layers = [hg.InfiniteAtmosphericLayer(grid, hg.Cn_squared_from_fried_parameter(0.15, 500e-9), L0=20,
                                          velocity=v, seed=3 + i, dtype=dtype)
              for i, v in enumerate(((10.0, 0.0), (-7.5, 13.0), (0.0, -31.0)))]
    atm = hg.MultiLayerAtmosphere(layers)
    for f in range(6):
        atm.evolve_until(0.011 * (f + 1))
    out[name] = atm.combined_screen().double().cpu().numpy()
# blocked transpose, float32 and float64
rng = np.random.default_rng(4)
m = sp.random(3000, 201, density=0.05, random_state=6, format='csr')
g = rng.standard_normal((37, 3000))
for name, dtype in (('tr32', torch.float32), ('tr64', torch.float64)):
    basis = SparseBasis(m, torch.device('cuda'), dtype)
    out[name] = basis.apply_transpose(torch.from_numpy(g)).double().cpu().numpy()
# EFC step
dz = np.zeros(4096, bool)
dz[rng.choice(4096, 700, replace=False)] = True
em = rng.standard_normal((203, 1400))
e = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
a = rng.standard_normal(203)
out['efc'] = hg.efc_step(em, e, dz, a, 0.3).cpu().numpy()
np.savez(sys.argv[1], **out)
'''


def _run(path, env_extra):
    env = dict(os.environ, **env_extra)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run([sys.executable, '-c', _CHILD, path, root], env=env, check=True, timeout=600)
    return np.load(path)


def test_one_cta_forms_match_the_cluster_forms(tmp_path):
    with_clusters = _run(str(tmp_path / 'a.npz'), {'HX_NO_CLUSTERS': '0'})
    without = _run(str(tmp_path / 'b.npz'), {'HX_NO_CLUSTERS': '1'})
    for name, tol in (('atm32', 1e-6), ('atm64', 1e-13), ('tr32', 1e-6), ('tr64', 1e-13), ('efc', 1e-13)):
        a, b = with_clusters[name], without[name]
        assert a.shape == b.shape
        err = np.linalg.norm(a - b) / np.linalg.norm(a)
        assert err < tol, (name, err)
