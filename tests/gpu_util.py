"""Helpers for the GPU tests: render through the C ABI into torch device
buffers and through the CPU oracle, in the same image layout."""
import numpy as np
import torch

TRACE_BYTES = 56


def gpu_exact(pkg, dev, tree, rec, cam, W, H, scales_inverted=False):
    """Plain (oracle-matching) kernel with traces.  Returns rgb (H,W,3) in the
    reference framebuffer layout (rows flipped), alpha (H,W), depth (H,W) and
    the trace records in kernel row order."""
    import oracle as O
    scene = pkg.renderer.Scene(tree, rec, scales_inverted=scales_inverted)
    rgb = torch.full((W * H * 3,), -1.0, device=dev)
    alpha = torch.full((W * H,), -1.0, device=dev)
    depth = torch.full((W * H,), -1.0, device=dev)
    tr = torch.zeros(W * H * TRACE_BYTES, dtype=torch.uint8, device=dev)
    scene.render_trace(cam, W, H, rgb, alpha, depth, tr)
    torch.cuda.synchronize()
    assert scene.status() == 0
    scene.close()
    trace = np.frombuffer(tr.cpu().numpy().tobytes(), dtype=O.TRACE_DTYPE)
    return (rgb.cpu().numpy().reshape(H, W, 3), alpha.cpu().numpy().reshape(H, W),
            depth.cpu().numpy().reshape(H, W), trace)


def oracle_image(O, tree, rec, cam, W, H, precision="f32", pixels=None, threads=0):
    S = O.OracleScene(tree.nodes, tree.offsets, tree.aabb, O.invert_scales(rec))
    rgb, a, d, tr = O.render(S, cam, W, H, pixels=pixels, precision=precision, trace=(precision == "f32"),
                             threads=threads)
    if pixels is not None:
        return rgb, a, d, tr
    return O.to_image(rgb, W, H), O.to_image(a, W, H), O.to_image(d, W, H), tr


def flipped_index(pixels, W, H):
    """Kernel pixel index y*W+x -> framebuffer index (H-1-y)*W+x."""
    y = pixels // W
    x = pixels % W
    return (H - 1 - y) * W + x
