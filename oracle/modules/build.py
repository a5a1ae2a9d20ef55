"""Build the CPU harness around the reference's module host code (test
infrastructure only): each module's main.c compiled unmodified from the vkdt
tree into oracle/_ref/mod_<name>.so, and oracle/modules/harness.c with the
tree's src/pipe/connector.c into oracle/_ref/libvkdt_modharness.so, against
the type-only shim in oracle/modules/shim. Needs the vkdt tree
(VKDT_REFERENCE); builds nothing without it."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "_ref")
TREE = os.environ.get("VKDT_REFERENCE", "/root/reference")
SRC = os.path.join(TREE, "src")
MODULES_DIR = os.path.join(SRC, "pipe", "modules")
CHAIN = ["denoise", "hilite", "demosaic", "crop", "colour", "filmcurv", "llap"]
EXTRA = ["nprof"]   # modules driven on their own (write_sink)
HARNESS = os.path.join(REF, "libvkdt_modharness.so")


def flags():
    return ["-O1", "-fPIC", "-std=gnu11", "-D_GNU_SOURCE", "-w", "-I" + os.path.join(HERE, "shim"),
            "-I" + os.path.join(SRC, "pipe"), "-I" + SRC]


def available():
    return os.path.exists(HARNESS) and all(os.path.exists(os.path.join(REF, "mod_%s.so" % m)) for m in CHAIN + EXTRA)


def _stale(out, srcs):
    return not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in srcs)


def build(force=False):
    if not os.path.isdir(MODULES_DIR):
        return available()
    os.makedirs(REF, exist_ok=True)
    shim = os.path.join(HERE, "shim", "vulkan", "vulkan.h")
    jobs = []
    for m in CHAIN + EXTRA:
        out = os.path.join(REF, "mod_%s.so" % m)
        src = os.path.join(MODULES_DIR, m, "main.c")
        if force or _stale(out, [src, shim]):
            jobs.append(["gcc"] + flags() + ["-shared", "-o", out, src, "-lm"])
    hsrc = [os.path.join(HERE, "harness.c"), os.path.join(SRC, "pipe", "connector.c")]
    if force or _stale(HARNESS, hsrc + [shim]):
        jobs.append(["gcc"] + flags() + ["-shared", "-o", HARNESS] + hsrc + ["-ldl", "-lm"])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    for j, p in procs:
        out = p.communicate()[0].decode()
        if p.returncode:
            raise RuntimeError("module harness build failed: %s\n%s" % (" ".join(j), out))
    return available()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
