"""A frame of a multi-volume fusion loop captured in one CUDA graph: depth
maps, the integration of the frame into several volumes of uneven sizes
(device-resident pose), and one batched extraction of all of them into
preallocated buffers.  Replaying the graph per frame gives the same volumes,
per-volume counts and soups as eager calls, also after an eager batched
call on the same context between replays (the graph keeps its own staging of
the volume table).

Reference counterpart: the per-volume loop of mc.run over a frame's volumes
(cu_kinect_fusion_v1.cu:3511-3737), integrate kf.cu:427-532."""
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu

# (nx, ny, nz): rows of 37, 71 and 45 voxels are not 16-byte multiples, so
# those volumes take the per-voxel tile fill instead of TMA
SIZES = [(37, 52, 40), (64, 64, 64), (71, 33, 50), (96, 80, 72), (45, 45, 91)]
EXTENT, W, H, F = 3.0, 160, 120, 131.25


def _frames(n):
    scene = synthetic.FusionScene(seed=8, extent=EXTENT)
    out = []
    for i in range(n):
        R, t = scene.pose(i, n)
        d = synthetic.mm_to_u16_bits(scene.depth_frame(R, t, w=W, h=H, fx=F, fy=F, cx=(W - 1) / 2,
                                                       cy=(H - 1) / 2, seed=40 + i, device="cuda"))
        out.append((d, R, t))
    return out


def _run(mcg, frames, graph, interleave=False):
    ctx = mcg.Context()
    k = mcg.intrinsic(F, F, (W - 1) / 2, (H - 1) / 2)
    vols = []
    for (nx, ny, nz) in SIZES:
        g = EXTENT / max(nx, ny, nz)
        vols.append(mcg.voxel_new((nx, ny, nz), 3 * g, 3 * g, g, ctx=ctx))
    cells = [v.grid_s for v in vols]
    caps = [12 * (nx * ny + ny * nz + nx * nz) for (nx, ny, nz) in SIZES]
    outs = [{"soup": torch.zeros((c, 28), dtype=torch.uint8, device="cuda"),
             "normals": torch.zeros((c, 3), dtype=torch.float32, device="cuda")} for c in caps]
    d_in = torch.empty_like(frames[0][0])
    meter = torch.empty((H, W), dtype=torch.float32, device="cuda")
    pose = torch.empty(12, dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()

    def frame():
        mcg.depth_to_maps(d_in, k, vertex=False, normal=False, ctx=ctx, stream=st, out_meter=meter)
        for v in vols:
            mcg.volumetric_integration_device_pose(v, k, pose, meter, ctx=ctx, stream=st)
        mcg.extract_batched_into([v.data for v in vols], cells, outs, caps, ctx=ctx, stream=st)

    saved = [v.data.clone() for v in vols]
    with torch.cuda.stream(st):
        # warm-up: sizes every buffer of the context; the volumes are restored
        d_in.copy_(frames[0][0])
        pose.copy_(mcg.extrinsic_tensor(frames[0][1], frames[0][2]))
        frame()
    torch.cuda.synchronize()
    for v, s0 in zip(vols, saved):
        v.data.copy_(s0)
    g = None
    if graph:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=st):
            frame()
        torch.cuda.synchronize()
        for v, s0 in zip(vols, saved):
            v.data.copy_(s0)
    results, side = [], []
    with torch.cuda.stream(st):
        for i, (d, R, t) in enumerate(frames):
            d_in.copy_(d)
            pose.copy_(mcg.extrinsic_tensor(R, t))
            if graph:
                g.replay()
            else:
                frame()
            st.synchronize()
            # the counts of a replay are read through the context's host state,
            # which an eager batched call in between makes that call's
            cnt = None
            if not (interleave and i > 1):
                cnt = mcg.counts_batched(ctx, len(vols))
                assert all(c["status"] == 0 for c in cnt)
            results.append((cnt, [(o["soup"].clone(), o["normals"].clone()) for o in outs]))
            if interleave and i == 1:
                # an eager batched call on the same context between replays
                # (a smaller batch: the context's device buffers keep their size)
                sub = [vols[2].data.clone(), vols[0].data.clone()]
                meshes = mcg.extract_batched(sub, [cells[2], cells[0]], ctx=ctx, stream=st)
                st.synchronize()
                side = list(zip(sub, [cells[2], cells[0]], meshes))
    torch.cuda.synchronize()
    return [v.data.clone() for v in vols], results, side


def test_batch_graph_replay_matches_eager(mcg):
    frames = _frames(4)
    ve, re, _ = _run(mcg, frames, graph=False)
    vg, rg, side = _run(mcg, frames, graph=True, interleave=True)
    for a, b in zip(ve, vg):
        assert torch.equal(a, b)
    nonempty = 0
    for (ce, be), (cg, bg) in zip(re, rg):
        # whole output buffers: the soups of every frame and what earlier
        # frames left beyond them
        for (se, ne), (sg, ng) in zip(be, bg):
            assert torch.equal(se, sg) and torch.equal(ne, ng)
        if cg is not None:
            assert [c["vertices"] for c in ce] == [c["vertices"] for c in cg]
        nonempty += sum(c["vertices"] > 0 for c in ce)
    assert nonempty >= 3 * len(SIZES)
    # the eager batch in between was itself right
    assert len(side) == 2
    for vol, cell, m in side:
        single = mcg.extract(vol, cell, soup=True, normals=True)
        torch.cuda.synchronize()
        assert single.counts["vertices"] == m.counts["vertices"] > 0
        assert torch.equal(single.soup, m.soup) and torch.equal(single.normals, m.normals)


def test_batch_graph_matches_single_extractions(mcg):
    frames = _frames(2)
    vols, res, _ = _run(mcg, frames, graph=True)
    cnt, bufs = res[-1]
    for v, c, (soup, nrm), (nx, ny, nz) in zip(vols, cnt, bufs, SIZES):
        n = c["vertices"]
        m = mcg.extract(v, EXTENT / max(nx, ny, nz), soup=True, normals=True)
        torch.cuda.synchronize()
        assert m.counts["vertices"] == n
        assert torch.equal(m.soup, soup[:n]) and torch.equal(m.normals, nrm[:n])
