"""Test infrastructure: copies the library's CUDA sources for a host build against the
emulation in tests/emu (used by tests/test_kernel_emulation.py and
tests/test_host_emulation.py).

- The dynamic shared-memory declaration becomes the emulated block's buffer.
- Every ``kernel<<<grid, block, smem, stream>>>(args);`` launch, and every call of the
  ``launch_k`` helper, becomes a call of ``emu::launch_kernel`` with the same
  configuration and a closure running the kernel.
- The size lists of the launch dispatch shrink to the sizes a test builds.
"""
import os
import re

SMEM_DECL = "extern __shared__ __align__(16) unsigned char smem_raw[];"
SMEM_EMU = "unsigned char* smem_raw = ::emu::t_blk->smem;"


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "(<[{":
            depth += 1
        elif ch in ")>]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def rewrite_launches(text):
    out, i = "", 0
    while True:
        j = text.find("<<<", i)
        if j < 0:
            return out + text[i:]
        k = max(text.rfind("\n", 0, j), text.rfind(";", 0, j), text.rfind("{", 0, j))
        name = text[k + 1:j].strip()
        e = text.find(">>>", j)
        cfg = _split_top(text[j + 3:e])
        if text[e + 3] != "(":
            raise ValueError("unexpected launch syntax near " + text[j - 40:e + 20])
        depth, m = 0, e + 3
        while True:
            if text[m] == "(":
                depth += 1
            elif text[m] == ")":
                depth -= 1
                if depth == 0:
                    break
            m += 1
        args = text[e + 4:m]
        smem = cfg[2] if len(cfg) > 2 else "0"
        strm = cfg[3] if len(cfg) > 3 else "0"
        clus = 2 if ("xyc_fused_kernel" in name or "mega_kernel" in name) else 1  # __cluster_dims__(2, 1, 1)
        out += (text[i:k + 1] + f"\n    ::emu::launch_kernel(dim3({cfg[0]}), dim3({cfg[1]}), (size_t)({smem}), "
                f"(cudaStream_t)({strm}), (const void*)(&{name}), {clus}, [=]() {{ {name}({args}); }})")
        i = m + 1


def rewrite_launch_k(text):
    """``launch_k(kernel, grid, block, smem, stream, args...)`` (the programmatic-launch
    helper of launch_impl.cuh) becomes the same ``emu::launch_kernel`` call as a
    triple-chevron launch; the helper's own definition is left alone."""
    out, i = "", 0
    while True:
        j = text.find("launch_k(", i)
        if j < 0:
            return out + text[i:]
        if text[max(0, j - 1)].isalnum() or text[max(0, j - 1)] == "_" or text[j:j + 22].startswith(
                "launch_k(void (*kern)"):
            out += text[i:j + 9]
            i = j + 9
            continue
        depth, m = 0, j + 8
        while True:
            if text[m] == "(":
                depth += 1
            elif text[m] == ")":
                depth -= 1
                if depth == 0:
                    break
            m += 1
        parts = _split_top(text[j + 9:m])
        name, grid, block, smem, strm, args = parts[0], parts[1], parts[2], parts[3], parts[4], parts[5:]
        clus = 2 if ("xyc_fused_kernel" in name or "mega_kernel" in name) else 1
        out += (text[i:j] + f"::emu::launch_kernel({grid}, {block}, (size_t)({smem}), (cudaStream_t)({strm}), "
                f"(const void*)(&{name}), {clus}, [=]() {{ {name}({', '.join(args)}); }})")
        i = m + 1


def copy_sources(csrc, out, sizes=None, launches=False):
    """Copies csrc/*.cu, *.cuh, *.h to out with the rewrites; returns how many
    shared-memory declarations were rewritten."""
    os.makedirs(out, exist_ok=True)
    n_decl = 0
    for f in os.listdir(csrc):
        if not f.endswith((".cu", ".cuh", ".h")):
            continue
        t = open(os.path.join(csrc, f)).read()
        n_decl += t.count(SMEM_DECL)
        t = t.replace(SMEM_DECL, SMEM_EMU)
        if sizes:
            xs = " ".join(f"X({n})" for n in sizes)
            for lst in ("CB_XY_SIZES", "CB_Z_SIZES", "CB_XYC_SIZES"):
                t = re.sub(rf"#define {lst}\(X\).*", f"#define {lst}(X) {xs}", t)
        if launches and "<<<" in t:
            t = rewrite_launches(t)
        if launches and "launch_k(" in t:
            # the helper's definition goes (every call of it becomes an emulated launch)
            t = re.sub(r"// \[launch_k definition\].*?// \[end launch_k definition\]", "", t, flags=re.S)
            t = rewrite_launch_k(t)
        with open(os.path.join(out, f), "w") as fh:
            fh.write(t)
    return n_decl
