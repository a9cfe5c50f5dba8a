"""The traversal's 4-wide tree (raymond_gb300/csrc/bvh_wide.cpp) on the CPU:
built from the reference's binary nodes (the golden BVH of 2,000 boxes and
the sphere field's), each wide node's child k carries exactly the box of the
binary node it stands for (the builder's collapse replayed here), empty
slots are marked, and the leaves cover every primitive range exactly once."""

import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "raymond_gb300", "csrc")

# Builds the wide tree and writes its 32 words per node.
DRIVER = r"""
#include <cstdio>
#include <cstdint>
#include <vector>
#include "bvh_wide.h"
int main(int argc, char** argv) {
    FILE* f = std::fopen(argv[1], "rb");
    std::vector<uint32_t> nodes;
    uint32_t w;
    while (std::fread(&w, 4, 1, f) == 1) nodes.push_back(w);
    std::fclose(f);
    std::vector<float> out;
    if (!rmd::build_wide_bvh(nodes.data(), uint32_t(nodes.size() / 8), out)) return 3;
    FILE* o = std::fopen(argv[2], "wb");
    std::fwrite(out.data(), 4, out.size(), o);
    std::fclose(o);
    return 0;
}
"""


@pytest.fixture(scope="module")
def builder(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("wide")
    src = d / "drv.cpp"
    src.write_text(DRIVER)
    exe = d / "drv"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(src),
                    os.path.join(CSRC, "bvh_wide.cpp"), "-o", str(exe)], check=True)

    def build(nodes):
        inp, out = d / "in.bin", d / "out.bin"
        np.ascontiguousarray(nodes, dtype=np.uint32).tofile(inp)
        r = subprocess.run([str(exe), str(inp), str(out)])
        assert r.returncode == 0
        return np.fromfile(out, dtype=np.uint32).reshape(-1, 32)

    return build


def check_tree(binary, wide):
    b = binary.reshape(-1, 8)
    bmin = b[:, 0:3].view(np.float32)
    bmax = b[:, 4:7].view(np.float32)
    first, count = b[:, 3], b[:, 7]
    # node: lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4], refs[4], spare[4]
    bounds = wide[:, 0:24].view(np.float32).reshape(-1, 6, 4)
    refs = wide[:, 24:28]

    ext = (bmax.astype(np.float64) - bmin).tolist()
    area = [e[0] * e[1] + e[1] * e[2] + e[2] * e[0] for e in ext]
    count_l, first_l = count.tolist(), first.tolist()
    # Walk both trees together: wide child k of node i stands for binary node c.
    stack = [(0, 0)]  # (wide node, binary node it covers)
    covered = np.zeros(len(first), dtype=np.int32)  # leaves reached, by binary index
    while stack:
        wi, bi = stack.pop()
        if count_l[bi] > 0:
            kids = [bi]
        else:
            # the builder's collapse: expand the inner child of largest area (first of equals)
            kids = [first_l[bi], first_l[bi] + 1]
            while len(kids) < 4:
                best, best_area = -1, -1.0
                for j, k in enumerate(kids):
                    if count_l[k] == 0 and area[k] > best_area:
                        best, best_area = j, area[k]
                if best < 0:
                    break
                f = first_l[kids[best]]
                kids[best] = f
                kids.append(f + 1)
        for k in range(4):
            ref = refs[wi, k]
            if k >= len(kids):
                assert ref == 0xFFFFFFFF
                assert np.all(bounds[wi, 0::2, k] == np.inf) and np.all(bounds[wi, 1::2, k] == -np.inf)
                continue
            c = kids[k]
            lo, hi = bounds[wi, 0::2, k], bounds[wi, 1::2, k]
            assert np.array_equal(lo, bmin[c]) and np.array_equal(hi, bmax[c]), (wi, k, lo, bmin[c], hi, bmax[c])
            if ref & 0x80000000:
                assert count[c] > 0 and (ref & 0xFFFFFF) == first[c] and ((ref >> 24) & 127) + 1 == count[c]
                covered[c] += 1
            else:
                stack.append((int(ref), int(c)))
    leaves = count > 0
    assert np.all(covered[leaves] == 1)


def test_golden_bvh_wide_tree_matches_binary(builder):
    g = np.load(os.path.join(HERE, "golden", "bvh_boxes.npz"))
    check_tree(g["nodes"], builder(g["nodes"]))


def test_sphere_field_wide_tree_matches_binary(builder):
    from raymond_gb300 import scenes

    scene, _, _ = scenes.sphere_field()
    nodes = scene.pack().nodes.reshape(-1)
    check_tree(nodes, builder(nodes))
