"""fn_particle_found's rule at each kind of evaluation point (ParticleFound,
L/Underworld/Function/src/ParticleFound.cpp:26-95): the swarm's own particles
are found; integration points are found where their element's particle map
found a particle of that swarm (id >= 0); plain coordinates and other swarms'
particles are not.  Host logic on CPU tensors; the GPU path is covered by
tests/test_zzz_gauss_swarm_gpu.py."""
import torch

from underworld2_gb300 import function as fn


class _Swarm:
    pass


def _ctx(pid):
    pid = torch.tensor(pid, dtype=torch.int64)
    return fn.EvalContext(pid, lambda: torch.zeros((pid.shape[0], 2), dtype=torch.float64), torch.device("cpu"))


def test_own_particles_found():
    s = _Swarm()
    pf = fn._ParticleFound(s)
    c = _ctx([0, 1, 2])
    c.swarm = s
    assert pf.evaluate_at(c).view(-1).tolist() == [1.0, 1.0, 1.0]
    c.swarm = _Swarm()
    assert pf.evaluate_at(c).view(-1).tolist() == [0.0, 0.0, 0.0]


def test_integration_points_follow_the_map():
    s = _Swarm()
    pf = fn._ParticleFound(s)
    c = _ctx([4, -1, 0, -1])
    c.map_swarm = s
    assert pf.evaluate_at(c).view(-1).tolist() == [1.0, 0.0, 1.0, 0.0]
    c.map_swarm = _Swarm()
    assert pf.evaluate_at(c).view(-1).tolist() == [0.0] * 4


def test_plain_coordinates_not_found():
    pf = fn._ParticleFound(_Swarm())
    assert pf.evaluate_at(_ctx([-1, -1])).view(-1).tolist() == [0.0, 0.0]
    assert pf._bool


def test_conditional_over_particle_found():
    s = _Swarm()
    pf = fn._ParticleFound(s)
    c = _ctx([3, -1])
    c.map_swarm = s
    f = fn.branching.conditional(((pf, 1.0), (True, 0.0)))
    assert f.evaluate_at(c).view(-1).tolist() == [1.0, 0.0]
