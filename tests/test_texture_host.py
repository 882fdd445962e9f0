"""Host logic of the hash-grid texture wrapper (CPU only; no kernel runs)."""
import pytest
import torch

from dmgs_gb300.build import build


@pytest.fixture(scope="module")
def texture_cls():
    build()
    from dmgs_gb300.texture import MLPTexture3D
    return MLPTexture3D


def test_aabb_host_copy_is_cached_and_refreshed(texture_cls):
    aabb = torch.tensor([[-1.0, -2.0, -3.0], [1.0, 2.0, 3.0]])
    tex = texture_cls(aabb, channels=48, device="cpu")
    h = tex._aabb_host()
    assert torch.equal(h, aabb) and h.dtype == torch.float32
    assert tex._aabb_host() is h                      # no copy while unchanged
    aabb.mul_(2.0)                                   # modified in place
    assert torch.equal(tex._aabb_host(), aabb)
    tex.AABB = torch.zeros(2, 3).index_fill_(0, torch.tensor([1]), 5.0)  # replaced
    assert torch.equal(tex._aabb_host(), tex.AABB)
    tex.AABB = [[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]]     # plain sequences work too
    assert tex._aabb_host().tolist() == [[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]]


def test_constructor_contract(texture_cls):
    aabb = torch.tensor([[-1.0] * 3, [1.0] * 3])
    tex = texture_cls(aabb, channels=27, device="cpu")
    assert sorted(tex.state_dict().keys()) == ["encoder.params", "net.net.0.weight",
                                               "net.net.2.weight", "net.net.4.weight"]
    assert tex.net.net[4].weight.shape == (27, 32)
    with pytest.raises(NotImplementedError):
        texture_cls(aabb, channels=5, device="cpu")
    with pytest.raises(NotImplementedError):
        texture_cls(aabb, channels=48, internal_dims=64, device="cpu")
