"""DIVeR decoder parameters: the torch-form layers and their packed layouts.

The decoder is the reference's pair of MLPs (model/diver.py:29-37,
model/mlps.py:21-30):
  mlp1: feature[C] -> hidden layers of width W -> (sigma, hidden[W])
  mlp2: (hidden[W], PE(view dir)[27]) -> W -> rgb[3], then sigmoid
with PE(d) = [d, sin(2^l pi d), cos(2^l pi d) for l in 0..3] (model/mlps.py:6-18).

DIVeR32: mlp_point = [32, 2, 33], mlp_view = [32, 1]
         (configs/nerf_synthetic_fine_diver32.py:118-127)
DIVeR64: mlp_point = [64, 1, 65], mlp_view = [64, 1]
         (configs/nerf_synthetic_fine.py:118-127)

Packed torch form ("plain" layout, float32), used by the FP32 kernels: each
Linear layer in order as W^T [in][out4] row-major (out4 = out rounded up to a
multiple of 4, extra columns zero) followed by its bias [out4], so every row
is a whole number of float4s.

Real-time form: the reference's `convert.py` folding and flat `params` array
(convert.py:59-140), see `pack_realtime`.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import torch

KINDS = {
    # kind: (width, mlp1 hidden layers)
    "diver32": (32, 2),
    "diver64": (64, 1),
}
PE_BANDS = 4
PE_DIM = 3 + 3 * 2 * PE_BANDS  # 27


@dataclass
class Decoder:
    kind: str
    channels: int
    layers: list = field(default_factory=list)  # [(weight [out,in], bias [out]), ...] mlp1 then mlp2

    @property
    def width(self) -> int:
        return KINDS[self.kind][0]

    @property
    def n_mlp1(self) -> int:
        return KINDS[self.kind][1] + 1

    def to(self, device) -> "Decoder":
        return Decoder(self.kind, self.channels, [(w.to(device), b.to(device)) for w, b in self.layers])

    def dims(self) -> list[tuple[int, int]]:
        return [(w.shape[1], w.shape[0]) for w, _ in self.layers]

    def state_dict(self) -> dict:
        """Names as in the reference's DIVeR module (mlp1.{0,2,4}, mlp2.{0,2})."""
        sd = {}
        for i, (w, b) in enumerate(self.layers[: self.n_mlp1]):
            sd[f"mlp1.{2 * i}.weight"], sd[f"mlp1.{2 * i}.bias"] = w, b
        for i, (w, b) in enumerate(self.layers[self.n_mlp1:]):
            sd[f"mlp2.{2 * i}.weight"], sd[f"mlp2.{2 * i}.bias"] = w, b
        return sd

    @staticmethod
    def from_state_dict(kind: str, sd: dict) -> "Decoder":
        width, depth = KINDS[kind]
        layers = [(sd[f"mlp1.{2 * i}.weight"], sd[f"mlp1.{2 * i}.bias"]) for i in range(depth + 1)]
        layers += [(sd[f"mlp2.{2 * i}.weight"], sd[f"mlp2.{2 * i}.bias"]) for i in range(2)]
        return Decoder(kind, layers[0][0].shape[1], [(w.float(), b.float()) for w, b in layers])


def layer_dims(kind: str, channels: int) -> list[tuple[int, int]]:
    width, depth = KINDS[kind]
    dims = [(channels, width)] + [(width, width)] * (depth - 1) + [(width, width + 1)]
    dims += [(width + PE_DIM, width), (width, 3)]
    return dims


def random_decoder(kind: str, channels: int, seed: int) -> Decoder:
    """Default nn.Linear initialisation (Kaiming-uniform, a=sqrt(5)) under manual_seed(seed), CPU."""
    g = torch.Generator().manual_seed(seed)
    layers = []
    for fin, fout in layer_dims(kind, channels):
        bound = 1.0 / math.sqrt(fin)
        # kaiming_uniform_(a=sqrt(5)) on [out, in] gives U(-1/sqrt(in), 1/sqrt(in))
        w = (torch.rand(fout, fin, generator=g) * 2 - 1) * bound
        b = (torch.rand(fout, generator=g) * 2 - 1) * bound
        layers.append((w, b))
    return Decoder(kind, channels, layers)


def pad4(n: int) -> int:
    return (n + 3) // 4 * 4


def plain_layout(kind: str, channels: int) -> list[tuple[int, int, int, int]]:
    """[(in, out, weight_offset, bias_offset)] of the packed torch form; rows are pad4(out) long."""
    out = []
    off = 0
    for fin, fout in layer_dims(kind, channels):
        w_off = off
        b_off = w_off + fin * pad4(fout)
        off = b_off + pad4(fout)
        out.append((fin, fout, w_off, b_off))
    return out


def plain_size(kind: str, channels: int) -> int:
    fin, fout, w_off, b_off = plain_layout(kind, channels)[-1]
    return b_off + pad4(fout)


def pack_plain(dec: Decoder) -> torch.Tensor:
    lay = plain_layout(dec.kind, dec.channels)
    flat = torch.zeros(plain_size(dec.kind, dec.channels), dtype=torch.float32)
    for (w, b), (fin, fout, w_off, b_off) in zip(dec.layers, lay):
        wt = torch.zeros(fin, pad4(fout))
        wt[:, :fout] = w.detach().float().cpu().t()
        flat[w_off:w_off + fin * pad4(fout)] = wt.reshape(-1)
        flat[b_off:b_off + fout] = b.detach().float().cpu()
    return flat


def unpack_plain_grad(kind: str, channels: int, flat: torch.Tensor) -> list[tuple[torch.Tensor, torch.Tensor]]:
    """Gradients in the packed layout -> [(dW [out,in], db [out])]."""
    res = []
    for fin, fout, w_off, b_off in plain_layout(kind, channels):
        dw = flat[w_off:w_off + fin * pad4(fout)].reshape(fin, pad4(fout))[:, :fout].t().contiguous()
        db = flat[b_off:b_off + fout].clone()
        res.append((dw, db))
    return res


# --- real-time form (convert.py) ---------------------------------------------

# Column order of the folded PE weights: per axis [d, sin x4, cos x4]
# (convert.py:89-92,128-131).
PE_REORDER = [0, 3, 9, 15, 21, 6, 12, 18, 24,
              1, 4, 10, 16, 22, 7, 13, 19, 25,
              2, 5, 11, 17, 23, 8, 14, 20, 26]
# flat params: 3168 floats for DIVeR32, 8288 for DIVeR64 over 32 channels
REALTIME_PARAMS = {"diver32": 3168, "diver64": 8288}


def pack_realtime(dec: Decoder) -> torch.Tensor:
    """The flat `params` array of the reference's serialized model
    (convert.py:63-140): the activation-free sigma/hidden layer is folded into
    mlp2's first layer, PE columns reordered, 28 zeros of padding.  DIVeR32's
    first layer (weightin) keeps only its bias here; its matrix is applied to
    the feature table at conversion time (`premultiply_features`)."""
    L = [(w.detach().float().cpu(), b.detach().float().cpu()) for w, b in dec.layers]
    W = dec.width
    if dec.kind == "diver32":
        (w01, b01), (w11, b11), (w21, b21), (w22, b22), (w3, b3) = L
        head = [b01]
        mid = [torch.cat([b11[:, None], w11], 1).t().reshape(-1)]
    else:
        (w1, b1), (w21, b21), (w22, b22), (w3, b3) = L
        head = []
        mid = [torch.cat([b1[:, None], w1], 1).t().reshape(-1)]
    lin40, bias40 = w21[:1], b21[:1]
    lin41 = w22[:, :W] @ w21[1:]
    bias41 = w22[:, :W] @ b21[1:] + b22
    lin42 = w22[:, W:]
    lin4 = torch.cat([lin40, lin41], 0)
    bias4 = torch.cat([bias40, bias41], 0)
    weight1 = torch.cat([bias4[0, None], lin4[0]], 0)
    w2 = torch.cat([bias4[1:, None], lin4[1:], lin42], 1)
    w2 = torch.cat([w2[:, :-PE_DIM], w2[:, -PE_DIM:][:, PE_REORDER]], -1)
    weight3 = torch.cat([b3[:, None], w3], -1)
    params = torch.cat(head + mid + [weight1.reshape(-1), w2.t().reshape(-1), weight3.t().reshape(-1), torch.zeros(28)], 0)
    expect = (32 + 33 * 32 + 33 + 60 * 32 + 33 * 3 + 28) if dec.kind == "diver32" else \
        ((1 + dec.channels) * 64 + 65 + 92 * 64 + 65 * 3 + 28)
    assert params.numel() == expect, params.numel()
    return params.contiguous()


def premultiply_features(dec: Decoder, features: torch.Tensor) -> torch.Tensor:
    """DIVeR32 stores features already multiplied by its first layer's matrix
    (convert.py:148-150); DIVeR64 stores them as they are."""
    if dec.kind == "diver32":
        w01 = dec.layers[0][0].to(features.device, torch.float32)
        return (features @ w01.t()).contiguous()
    return features.contiguous()


# --- tensor-core operand image -------------------------------------------------

def _kmajor_index(N: int, K: int) -> torch.Tensor:
    """Element offsets of an [N][K] 16-bit tile in the K-major, no-swizzle
    core-matrix layout the tcgen05 kernels read: 8x8 blocks of 128 contiguous
    bytes, block (n/8, k/8) at ((n/8) * (K/8) + k/8) * 64 elements."""
    n = torch.arange(N)[:, None]
    k = torch.arange(K)[None, :]
    return (((n // 8) * (K // 8) + k // 8) * 64 + (n % 8) * 8 + (k % 8)).reshape(-1)


def tc_matrices(dec: Decoder):
    """The decoder as the tensor-core kernel's layer list [(W [N][K], bias [N])]:
    mlp1 hidden layers; mlp1's output layer with the hidden rows first and the
    sigma row at index `width` (N padded to width + 16); the hidden-input part
    of mlp2's first layer (its bias and PE part are added per ray in FP32);
    mlp2's output layer (N padded to 16)."""
    W = dec.width
    d1 = dec.n_mlp1 - 1
    L = [(w.detach().float().cpu(), b.detach().float().cpu()) for w, b in dec.layers]
    mats = [L[l] for l in range(d1)]
    w, b = L[d1]
    wo = torch.zeros(W + 16, W)
    bo = torch.zeros(W + 16)
    wo[:W], wo[W] = w[1:], w[0]
    bo[:W], bo[W] = b[1:], b[0]
    mats.append((wo, bo))
    w, b = L[d1 + 1]
    mats.append((w[:, :W].clone(), torch.zeros(W)))
    w, b = L[d1 + 2]
    w4 = torch.zeros(16, W)
    b4 = torch.zeros(16)
    w4[:3], b4[:3] = w, b
    mats.append((w4, b4))
    return mats


def _kmajor_images(mats, dt) -> tuple[list[torch.Tensor], list[tuple[int, int, int]]]:
    """Each [N][K] matrix as a flat K-major core-matrix image of dtype dt, with
    its (byte offset of a 2-byte element image, K, N)."""
    images, table, off = [], [], 0
    for m in mats:
        N, K = m.shape
        img = torch.zeros(N * K, dtype=dt)
        img[_kmajor_index(N, K)] = m.reshape(-1).to(dt)
        images.append(img)
        table.append((off, K, N))
        off += N * K * 2
    return images, table


def pack_tc(dec: Decoder, bf16: bool = True):
    """(blob uint8 [bytes], bias float32, layers int32 [n, 4] = (byte offset, K, N, bias offset))."""
    dt = torch.bfloat16 if bf16 else torch.float16
    mats = tc_matrices(dec)
    images, table = _kmajor_images([w for w, _ in mats], dt)
    boffs = [0]
    for _, b in mats[:-1]:
        boffs.append(boffs[-1] + b.numel())
    rows = [[off, K, N, bo] for (off, K, N), bo in zip(table, boffs)]
    return (torch.cat([i.view(torch.uint8) for i in images]), torch.cat([b for _, b in mats]).float(),
            torch.tensor(rows, dtype=torch.int32))


def tc_bwd_matrices(dec: Decoder):
    """Transposed weights for the tensor-core backward (DIVeR32): per layer
    W^T as [N = in][K = out padded to 16], the mlp1 output layer in the torch
    order (sigma first), so delta @ W^T gives the input gradient."""
    if dec.kind != "diver32":
        raise ValueError("the tensor-core backward is implemented for DIVeR32")
    W = dec.width
    (w0, _), (w1, _), (w2, _), (w3, _), (w4, _) = [(w.detach().float().cpu(), b) for w, b in dec.layers]
    m2 = torch.zeros(W, W + 16)
    m2[:, :W + 1] = w2.t()
    m4 = torch.zeros(W, 16)
    m4[:, :3] = w4.t()
    return [w0.t().contiguous(), w1.t().contiguous(), m2, w3[:, :W].t().contiguous(), m4]


def pack_tc_bwd(dec: Decoder, bf16: bool = True):
    """(blob uint8, layers int32 [n, 3] = (byte offset, K, N)) of tc_bwd_matrices."""
    dt = torch.bfloat16 if bf16 else torch.float16
    images, table = _kmajor_images(tc_bwd_matrices(dec), dt)
    return torch.cat([i.view(torch.uint8) for i in images]), torch.tensor(table, dtype=torch.int32)


def tc_index_maps(kind: str, channels: int) -> dict:
    """Where every element of the tensor-core images comes from in the packed
    plain parameter vector: index + 1, or 0 for padding.  The images are pure
    rearrangements of the parameters, so a gather of the (zero-prefixed)
    parameter vector rebuilds them on the device, e.g. after an optimizer step,
    without a host round trip.  Keys: 'fwd' (element indices of pack_tc's blob
    as 2-byte elements), 'bias', 'table' (pack_tc's layer rows), and for
    DIVeR32 over 32 channels 'bwd' / 'bwd_table' (pack_tc_bwd)."""
    n = plain_size(kind, channels)
    ids = torch.arange(1, n + 1, dtype=torch.float32)  # exact in float32 (n < 2^24)
    dec = Decoder(kind, channels, unpack_plain_grad(kind, channels, ids))
    mats = tc_matrices(dec)
    images, _ = _kmajor_images([w for w, _ in mats], torch.float32)
    _, _, table = pack_tc(dec, True)
    out = {"fwd": torch.cat(images).long(), "bias": torch.cat([b for _, b in mats]).long(), "table": table}
    if kind == "diver32" and channels == 32:
        bim, btab = _kmajor_images(tc_bwd_matrices(dec), torch.float32)
        out["bwd"] = torch.cat(bim).long()
        out["bwd_table"] = torch.tensor(btab, dtype=torch.int32)
    return out
