"""GPU: fixed-capacity segments (device-held counts) and the CUDA-graph
training step / render against the eager pipeline.

Tolerances (stated): capacity-mode segments are bit-identical to the exact
ones; graph-replayed loss equals the eager loss within 1e-6 relative and the
gradients within 1e-5 relative to their largest magnitude (the grid gradient
is accumulated with atomics, whose order differs between runs); rendered rgb
of a replay within 1e-6 abs of the eager render."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def small_field(active=True):
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    if active:
        sc.decoder.layers[sc.decoder.n_mlp1 - 1][1][0] += 0.6  # density above zero
    return sc, DIVeRField.from_scene(sc, "cuda")


def rays(n, seed):
    from diver_gb300 import scenes

    o, d = scenes.small_view("cuda", seed_offset=seed)
    g = torch.Generator().manual_seed(seed)
    pick = torch.randperm(o.shape[0], generator=g)[:n].cuda()
    return o[pick].contiguous(), d[pick].contiguous()


def test_capacity_segments_match_exact():
    sc, field = small_field()
    o, d = rays(3000, 1)
    exact = field.segments(o, d)
    cap = field.segments(o, d, capacity=field.segment_capacity(o.shape[0]))
    S = exact.total
    assert cap.total == field.segment_capacity(o.shape[0]) >= S
    assert cap.max_count is None and int(cap.max_dev.item()) == exact.max_count
    assert torch.equal(cap.offsets, exact.offsets)
    assert torch.equal(cap.seg[:S], exact.seg)
    assert torch.equal(cap.t[:S], exact.t)
    assert torch.equal(cap.ray[:S], exact.ray)
    with pytest.raises(ValueError):
        field.segments(o, d, capacity=S)


def _eager(field, o, d, tgt, form):
    rgb, reg = field(o, d, form=form)
    loss = torch.nn.functional.mse_loss(rgb, tgt) + 1e-5 * reg
    gv, gp = torch.autograd.grad(loss, [field.voxels, field.params])
    return loss.detach(), gv, gp


def _close(a, b, rel):
    scale = max(a.abs().max().item(), 1e-30)
    return (a - b).abs().max().item() <= rel * scale


@pytest.mark.parametrize("form", ["fp32", "bf16"])
def test_train_step_graph_matches_eager(form):
    from diver_gb300.graphs import TrainStepGraph

    sc, field = small_field()
    batches = []
    for k in range(3):
        o, d = rays(2048, 10 + k)
        batches.append((o, d, torch.rand(o.shape[0], 3, generator=torch.Generator().manual_seed(k)).cuda()))
    step = TrainStepGraph(field, *batches[0], form=form)
    for o, d, tgt in batches[1:] + batches[:1]:
        loss, gv, gp = step(o, d, tgt)
        loss, gv, gp = loss.clone(), gv.clone(), gp.clone()
        el, egv, egp = _eager(field, o, d, tgt, form)
        torch.cuda.synchronize()
        assert abs(loss.item() - el.item()) <= 1e-6 * abs(el.item())
        assert _close(egv, gv, 1e-5)
        assert _close(egp, gp, 1e-5)


def test_train_step_graph_sees_parameter_updates():
    from diver_gb300.graphs import TrainStepGraph

    sc, field = small_field()
    o, d = rays(2048, 20)
    tgt = torch.rand(o.shape[0], 3, generator=torch.Generator().manual_seed(5)).cuda()
    step = TrainStepGraph(field, o, d, tgt, form="bf16")
    with torch.no_grad():
        field.params.mul_(0.9)  # an in-place update, as an optimizer makes
        field.voxels.add_(0.01)
    loss, gv, gp = step(o, d, tgt)
    loss, gv, gp = loss.clone(), gv.clone(), gp.clone()
    el, egv, egp = _eager(field, o, d, tgt, "bf16")
    assert abs(loss.item() - el.item()) <= 1e-6 * abs(el.item())
    assert _close(egp, gp, 1e-5)


@pytest.mark.parametrize("form", ["fp32", "bf16"])
def test_render_graph_matches_eager(form):
    from diver_gb300.graphs import RenderGraph

    sc, field = small_field()
    o, d = rays(4096, 30)
    rg = RenderGraph(field, o, d, form=form)
    o2, d2 = rays(4096, 31)
    got = rg(o2, d2).clone()
    with torch.no_grad():
        ref, _ = field(o2, d2, form=form)
    assert (got - ref).abs().max().item() <= 1e-6
