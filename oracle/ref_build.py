"""TEST INFRASTRUCTURE ONLY: build the reference itself (Sinchanrc/Beach-Slope,
Fortran 2008) into oracle/_ref/, in an image without a Fortran compiler.

Recipe:
1. read the reference's compiled source files (exec.sh:19-30, minus
   output.f90, whose writers the driver does not call) from the reference
   tree;
2. apply the patch that takes Intel MKL out, as a text substitution on the
   in-memory copy (nothing is written back, nothing is copied into the
   repository):
   * initialize.f90: the MKL `include` lines, `use mkl_pardiso` and the
     PARDISO handle array (initialize.f90:1-5, 13, 71-74);
   * solver.f90: the MKL-based `fgmres`, `fgmres_mkl` and `pardisosolver`
     (solver.f90:306-540);
   * isph.f90: `ppesolve` calls the reference's own CSR conversion and
     BiCGStab -- the call the reference keeps commented out (isph.f90:460-461)
     -- in place of `call fgmres`, after allocating the CSR value and column
     arrays that only that path uses (finmax rows of the ELL width
     ceiling(fac2*fplistmax), memory.f90:138);
   * solver.f90 `bicgstab`: the stopping test on the relative change of the
     iterate (itls = 1e-2, solver.f90:233-242) becomes a test on the
     recurrence residual, ||r|| <= 1e-13 ||b||, capped at 20000 iterations,
     so that the pressure is the solution of the assembled system to
     rounding (the reference's own test stops at a loose, iterate-dependent
     point, which no second implementation can reproduce);
3. translate the modules to C++ with oracle/ref_translate.py;
4. compile them with oracle/ref_driver.cpp (the driver: main.f90's set-up
   and first phase, state dumps) into oracle/_ref/ref_main.

    python oracle/ref_build.py [reference root]
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = "/root/reference"
FILES = ["particle", "interactions", "transfer", "domain", "initialize", "kernel", "functions", "search",
         "gradient", "setup", "solver", "boundary", "internal", "memory", "isph", "integrator", "turbulence",
         "part_shift", "qsort", "scalar", "porous"]


def _sub(text, pattern, repl, count=1, flags=re.S):
    new, n = re.subn(pattern, repl, text, count=count, flags=flags)
    if n == 0:
        raise RuntimeError(f"patch pattern not found: {pattern[:60]!r}")
    return new


def patched_sources(root=REF):
    src = {}
    for f in FILES:
        with open(os.path.join(root, f + ".f90")) as fh:
            src[f] = fh.read()
    t = src["initialize"]
    t = _sub(t, r"^include\s+['\"]mkl_[^'\"]*['\"]\s*$", "", count=0, flags=re.M | re.I)
    t = _sub(t, r"^\s*use\s+mkl_pardiso\s*$", "", flags=re.M | re.I)
    t = _sub(t, r"^\s*type\s*\(\s*MKL_PARDISO_HANDLE\s*\)\s*::.*$", "", flags=re.M | re.I)
    src["initialize"] = t
    t = src["solver"]
    t = _sub(t, r"\n\s*subroutine\s+fgmres\s*\(\s*\).*?(?=\nend\s+module)", "\n", flags=re.S | re.I)
    t = _sub(t, r"\n(\s*)do\s+ks\s*=\s*1\s*,\s*ls\s*\n\s*if\s*\(\s*abs\(real\(\(sl\(ks\)-guess\(ks\)\),dp\)"
                r".*?end\s+do\s*\n",
             "\n\\1tcal=0\n\\1if ((sqrt(vecvec(ls,rs,rs))>1e-13_dp*sqrt(vecvec(ls,bvecs,bvecs))).and.(n<20000)) tcal=1\n"
             "\\1guess=sl\n", flags=re.S | re.I)
    src["solver"] = t
    t = src["isph"]
    t = _sub(t, r"^(\s*)call\s+fgmres\s*$",
             "\\1if (.not.allocated(fval)) allocate(fval(finmax*ceiling(fac2*fplistmax)),"
             "fcol(finmax*ceiling(fac2*fplistmax)))\n"
             "\\1call format(fmatrix,fval,frow,fcol,finmax)\n\\1call bicgstab(tl,fguess,finmax,fval,frow,fcol,fvec,fsol)",
             flags=re.M | re.I)
    src["isph"] = t
    return [(f + ".f90", src[f]) for f in FILES]


def build(root=REF, verbose=False):
    sys.path.insert(0, HERE)
    import ref_translate
    os.makedirs(OUT, exist_ok=True)
    cpp = ref_translate.translate_files(patched_sources(root))
    gen = os.path.join(OUT, "ref_modules.cpp")
    with open(gen, "w") as f:
        f.write(cpp)
    exe = os.path.join(OUT, "ref_main")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", "-include", gen,
           os.path.join(HERE, "ref_driver.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compiling the translated reference failed:\n" + r.stderr[-4000:])
    if verbose:
        print(exe)
    return exe


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else REF, verbose=True)
