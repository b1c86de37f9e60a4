"""Build the reference program from its own sources for one configuration.

TEST INFRASTRUCTURE ONLY.  The reference (caravangelo/inflation-easy) fixes N
and its feature switches at compile time in src/parameters.h.  This recipe
compiles the .cpp files where they lie in the read-only reference tree.  Only
parameters.h is patched, with the compile-time lines set (the same regex
patching the reference's own tests/regression_main_n16.py:71-76 does).  The
patched copy goes to a temporary folder beside symbolic links to the other
source files; g++ compiles through the links, so a quoted include resolves in
that folder and finds the patched header.  The build uses the reference Makefile's flags plus
-ffp-contract=off (IEEE evaluation, so the x86 and Arm builds agree) and links
oracle/ref_driver.cpp, which runs the unmodified main() and dumps state.  Only
the binary is kept, in the git-ignored oracle/_ref/<tag>/.

Nothing here is shipped or used by the product; only tests and the golden
fixture generator call it, and only where the reference tree is present.

    python oracle/build_ref.py --N 16 --numerical 0 --sigw 0 --deltaN 1 [--post 1]
"""
from __future__ import annotations

import argparse
import os
import re
import shutil
import subprocess
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("IE_REFERENCE_ROOT", "/root/reference"))


def ref_available() -> bool:
    return (REF_ROOT / "src" / "evolution.cpp").is_file()


def tag_for(N: int, numerical: int, sigw: int, deltaN: int, post: int = 0) -> str:
    return f"n{N}_{'usr' if numerical else 'hill'}_sigw{sigw}_dn{deltaN}" + ("_post1" if post else "")


def build(N: int, numerical: int, sigw: int, deltaN: int, jobs: int = 8, post: int = 0) -> Path:
    """Returns the path of the built driver binary (cached by configuration).
    post = 1 keeps the reference's post-inflation phase (src/parameters.h:31),
    which needs SIGW on."""
    if not ref_available():
        raise FileNotFoundError(f"reference sources not found under {REF_ROOT}")
    tag = tag_for(N, numerical, sigw, deltaN, post)
    out = HERE / "_ref" / tag
    exe = out / "ie_ref"
    if exe.is_file() and exe.stat().st_mtime >= (HERE / "ref_driver.cpp").stat().st_mtime:
        return exe
    ref_src = REF_ROOT / "src"
    if (out / "src").exists():   # source copies left by an older version of this recipe
        shutil.rmtree(out / "src")
    out.mkdir(parents=True, exist_ok=True)
    txt = (ref_src / "parameters.h").read_text()
    subs = [
        (r"#define numerical_potential \d+", f"#define numerical_potential {numerical}"),
        (r"#define perform_deltaN \d+", f"#define perform_deltaN {deltaN}"),
        (r"#define calculate_SIGW \d+", f"#define calculate_SIGW {sigw}"),
        (r"#define post_inflation \d+", f"#define post_inflation {post}"),
        (r"const int N = \d+;", f"const int N = {N};"),
    ]
    for pat, rep in subs:
        txt, n = re.subn(pat, rep, txt, count=1)
        if n != 1:
            raise RuntimeError(f"could not patch {pat!r} in parameters.h")
    with tempfile.TemporaryDirectory(prefix="ie_ref_src_") as tmp:
        lnk = Path(tmp)
        for f in ref_src.iterdir():
            if f.name != "parameters.h":
                os.symlink(f, lnk / f.name)
        (lnk / "parameters.h").write_text(txt)
        flags = ["-std=c++17", "-O3", "-DNDEBUG", "-ffp-contract=off", "-fopenmp", f"-I{lnk}"]
        objs = []
        procs = []
        for cpp in sorted(lnk.glob("*.cpp")):
            obj = out / (cpp.stem + ".o")
            extra = ["-Dmain=ie_ref_main"] if cpp.name == "main.cpp" else []
            procs.append(subprocess.Popen(["g++", *flags, *extra, "-c", str(cpp), "-o", str(obj)],
                                          stderr=subprocess.PIPE, text=True))
            objs.append(str(obj))
        drv = out / "ref_driver.o"
        procs.append(subprocess.Popen(["g++", *flags, "-c", str(HERE / "ref_driver.cpp"), "-o", str(drv)],
                                      stderr=subprocess.PIPE, text=True))
        objs.append(str(drv))
        errs = [(p, p.communicate()[1]) for p in procs]
        bad = [e for p, e in errs if p.returncode != 0]
        if bad:
            raise RuntimeError("reference compilation failed:\n" + bad[0][-2000:])
    wrap = (["-Wl,--wrap=_Z4savei"] + (["-Wl,--wrap=_Z5saveNv"] if deltaN else []) +
            (["-Wl,--wrap=_Z19save_post_inflationi"] if post else []))
    subprocess.check_call(["g++", "-fopenmp", *wrap, *objs, "-o", str(exe), "-lm"])
    for o in objs:
        os.unlink(o)
    return exe


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, required=True)
    ap.add_argument("--numerical", type=int, default=0)
    ap.add_argument("--sigw", type=int, default=0)
    ap.add_argument("--deltaN", type=int, default=1)
    ap.add_argument("--post", type=int, default=0)
    a = ap.parse_args()
    print(build(a.N, a.numerical, a.sigw, a.deltaN, post=a.post))


if __name__ == "__main__":
    main()
