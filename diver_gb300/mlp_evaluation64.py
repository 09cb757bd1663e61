"""Drop-in for utils/mlp_evaluation64 (DIVeR64 real-time decoder): `upload_weight`
and `mlp_eval` with the reference's arguments (utils/mlp_evaluation64/__init__.py:18-44)."""
from .realtime import mlp_eval as _mlp_eval
from .realtime import upload_weight as _upload


def upload_weight(device_id, params, voxel_map):
    return _upload(device_id, params, voxel_map, width=64)


def mlp_eval(rgba, coord, voxels, v, mask):
    return _mlp_eval(rgba, coord, voxels, v, mask, width=64)
