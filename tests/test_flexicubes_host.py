"""Host logic of the FlexiCubes wrapper (CPU only): recognising the three
cube weights as column slices of one [C, 21] tensor, the layout the
reference's stage 2 passes (scene/gaussian_geo_model_mlp_flex.py:246-247),
so that the kernels read and write it in place."""
import torch

from dmgs_gb300.flexicubes import _fused_weights

C = 37


def slices(W):
    return W[:, :12], W[:, 12:20], W[:, 20]


def test_column_slices_of_one_tensor_are_recognised():
    W = torch.randn(C, 21, requires_grad=True)
    assert _fused_weights(*slices(W), C) is W
    # a non-leaf producer (e.g. a network's output) works the same way
    V = W * 2
    assert _fused_weights(*slices(V), C) is V


def test_other_layouts_fall_back():
    W = torch.randn(C, 21)
    b, a, g = slices(W)
    assert _fused_weights(b.clone(), a, g, C) is None            # separate tensors
    assert _fused_weights(b, a, None, C) is None                 # a weight missing
    assert _fused_weights(W[:, 1:13], W[:, 13:21], W[:, 0], C) is None  # other columns
    assert _fused_weights(*slices(W.double()), C) is None        # not float32
    assert _fused_weights(*slices(W), C + 1) is None             # wrong cube count
    Wide = torch.randn(C, 24)
    assert _fused_weights(Wide[:, :12], Wide[:, 12:20], Wide[:, 20], C) is None  # row stride 24
    Wt = torch.randn(21, C).t()                                   # not contiguous
    assert _fused_weights(Wt[:, :12], Wt[:, 12:20], Wt[:, 20], C) is None
