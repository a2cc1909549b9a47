"""Every kernel the library launches chained to its stream's previous kernel (programmatic
dependent launch, `launch_chained`) waits for that kernel before it touches memory: its
first statement is `chain_enter()`. A chained kernel without it would read the previous
kernel's outputs while they are still being written. Checked on the sources, so it needs
no GPU."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "surface_match_gb300", "csrc")


def _sources():
    files = glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    return {f: open(f).read() for f in files}


def _first_statement(src, kernel):
    m = re.search(r"__global__[^{;]*?\b" + kernel + r"\s*\(", src)
    if not m:
        return None
    body = src[src.index("{", m.end()) + 1:]
    for line in body.split("\n"):
        line = line.strip()
        if line and not line.startswith("//"):
            return line
    return None


def test_chained_kernels_wait_before_touching_memory():
    src = _sources()
    everything = "\n".join(src.values())
    chained = set()
    for text in src.values():
        chained.update(re.findall(r"launch_chained\(\s*\w+\s*,\s*(\w+)", text))
    assert len(chained) >= 40  # sampler, scans, grids, normals, voting, clustering, refinement
    for k in sorted(chained):
        first = _first_statement(everything, k)
        assert first is not None, f"kernel {k} not found"
        assert re.match(r"(smd::)?chain_enter\(\);", first), f"{k} starts with: {first}"


def test_every_hot_path_launch_is_chained():
    # the single-scene path's kernels in these files are all launched through launch_chained
    # (a plain <<<...>>> launch there would go unnoticed by the check above)
    for name in ("icp.cu", "cluster.cu", "vote_pipe.cu"):
        text = open(os.path.join(CSRC, name)).read()
        plain = re.findall(r"(\w+)\s*(?:<[^<>]*>)?\s*<<<", text)
        allowed = {"k_init"}  # follows a memset: an ordinary launch
        assert set(plain) <= allowed, f"{name}: ordinary launches of {sorted(set(plain) - allowed)}"
