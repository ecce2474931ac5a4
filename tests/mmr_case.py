"""The three-surface multisurface study of the golden vectors (tm_func
in-memory bodies): an icosphere-3 mesh with a full mask, an icosphere-2 mesh
with masked-out vertices and a small voxel volume with the multimodal
26-neighbour lists.  Rebuilt from the fixture and the deterministic mesh
generator, for the oracle pins and the GPU drop-in tests alike."""
import numpy as np

from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import synth


def mmr_case(golden):
    va, fa = synth.icosphere(3)
    vb, fb = synth.icosphere(2)
    oa, ia = A.mesh_csr(fa, va.shape[0])
    ob, ib = A.mesh_csr(fb, vb.shape[0])
    masks = np.empty(3, dtype=object)
    masks[0] = np.ones((va.shape[0], 1, 1), bool)
    masks[1] = golden["mmr_mask_b"][:, None, None]
    masks[2] = golden["mmr_vol"]
    adjs = np.empty(3, dtype=object)
    for i, (o, x) in enumerate(((oa, ia), (ob, ib), (golden["mmr_adj_vol_off"], golden["mmr_adj_vol_idx"]))):
        lists = A.from_csr(o, x)
        arr = np.empty(len(lists), dtype=object)
        for j, l in enumerate(lists):
            arr[j] = list(l)
        adjs[i] = arr
    return {"masks": masks, "adjs": adjs, "y": golden["mmr_y"], "x": golden["mmr_x"],
            "pos": [int(p) for p in golden["mmr_pos"]], "full": golden["mmr_full"], "vd": golden["mmr_vd"],
            "perm": golden["mmr_perm"]}


def csv_values(text):
    return np.array([float(v) for v in str(text).split()])
