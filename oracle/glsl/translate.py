"""Compile the reference's GLSL compute shaders of the development path for
the CPU (test infrastructure only).

Reads the shader sources where they lie in the vkdt tree, resolves their
#includes, runs the C preprocessor, rewrites the GLSL-only syntax to C++
(glsl.hpp provides the types and built-ins) and writes one translation unit
per shader into oracle/_ref/, which is then compiled into
oracle/_ref/libvkdt_ref.so. Nothing here is committed output: oracle/_ref/ is
a build directory.

Usage: python oracle/glsl/translate.py [path to vkdt/src/pipe/modules]
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
# the vkdt source tree (VKDT_REFERENCE, default: where this build found it)
DEFAULT_MODULES = os.path.join(os.environ.get("VKDT_REFERENCE", "/root/reference"), "src", "pipe", "modules")

# (module, kernel) of the development path
SHADERS = [
    ("denoise", "noop"), ("denoise", "half"), ("denoise", "downcov"), ("denoise", "down"),
    ("denoise", "assemble"), ("denoise", "doub"),
    ("hilite", "half"), ("hilite", "reduce"), ("hilite", "assemble"), ("hilite", "doub"),
    ("demosaic", "down"), ("demosaic", "gauss"), ("demosaic", "splat"), ("demosaic", "fix"),
    ("demosaic", "halfsize"), ("demosaic", "rcd_conv"), ("demosaic", "rcd_fill"), ("shared", "resample"),
    ("crop", "main"), ("lens", "main"), ("colour", "main"), ("filmcurv", "main"),
    ("llap", "curve"), ("llap", "reduce"), ("llap", "assemble"), ("llap", "colour"),
    ("i-mcraw", "decode"), ("colenc", "main"), ("grade", "main"), ("rawhist", "collect"), ("hist", "collect"),
]


def resolve_includes(path, moddir, seen_stack=()):
    """Inline #include "x" (searched beside the file, then in the modules dir),
    dropping #version and #extension lines."""
    out = []
    base = os.path.dirname(path)
    for line in open(path).read().split("\n"):
        s = line.strip()
        if s.startswith("#version") or s.startswith("#extension"):
            continue
        m = re.match(r'#\s*include\s+"([^"]+)"', s)
        if m:
            name = m.group(1)
            cand = [os.path.join(base, name), os.path.join(moddir, name)]
            f = next((c for c in cand if os.path.exists(c)), None)
            if f is None:
                raise RuntimeError("include %s not found from %s" % (name, path))
            if f in seen_stack:
                continue
            out.append(resolve_includes(f, moddir, seen_stack + (f,)))
            continue
        out.append(line)
    return "\n".join(out)


def cpp(text):
    r = subprocess.run(["g++", "-E", "-P", "-x", "c++", "-DGL_core_profile=1", "-"], input=text,
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError("preprocessor failed:\n" + r.stderr)
    return r.stdout


def replace_array_ctors(s):
    """TYPE[](a, b, ...) -> {a, b, ...}"""
    while True:
        m = re.search(r"\b\w+\s*\[\s*\]\s*\(", s)
        if not m:
            return s
        i = m.end()
        depth = 1
        j = i
        while depth:
            if s[j] == "(":
                depth += 1
            elif s[j] == ")":
                depth -= 1
            j += 1
        s = s[:m.start()] + "{" + s[i:j - 1] + "}" + s[j:]


STD140_ALIGN = {"vec4": 16, "ivec4": 16, "uvec4": 16, "mat3": 16, "vec3": 16, "ivec3": 16, "uvec3": 16,
                "vec2": 8, "ivec2": 8, "uvec2": 8}


def scalar_swizzles(text):
    """GLSL allows .x on a scalar: inside each function body, NAME.x of a
    variable or parameter declared float becomes NAME."""
    out, pos = [], 0
    for m in re.finditer(r"^[\w ]+?\b(\w+)\s*\(([^;{}]*)\)\s*\{", text, flags=re.M):
        if m.start() < pos:
            continue
        depth, j = 1, m.end()
        while depth and j < len(text):
            depth += {"{": 1, "}": -1}.get(text[j], 0)
            j += 1
        body = text[m.start():j]
        names = set(re.findall(r"\bfloat\s+(\w+)", body))
        for n in names:
            body = re.sub(r"\b%s\.x\b" % n, n, body)
        out.append(text[pos:m.start()])
        out.append(body)
        pos = j
    out.append(text[pos:])
    return "".join(out)


VEC_TYPES = ("vec2", "vec3", "vec4", "ivec2", "ivec3", "ivec4", "uvec2", "uvec3", "uvec4")


def swizzle_overloads(text):
    """GLSL passes out/inout arguments by copy in / copy out, so a swizzle
    (xyY.xy) may be one. For every function with vector reference parameters
    add an overload per such parameter that takes a swizzle and copies."""
    extra = []
    for m in re.finditer(r"^(\w+)\s+(\w+)\s*\(([^;{}()]*)\)\s*\{", text, flags=re.M):
        ret, name, params = m.group(1), m.group(2), m.group(3)
        plist = [p.strip() for p in params.split(",") if p.strip()]
        for i, p in enumerate(plist):
            pm = re.match(r"(\w+)\s*&\s*(\w+)$", p)
            if not pm or pm.group(1) not in VEC_TYPES:
                continue
            t, pn = pm.group(1), pm.group(2)
            sig = list(plist)
            sig[i] = "swz<T_, N_, I_...> &%s" % pn
            args = [re.search(r"(\w+)$", q).group(1) for q in plist]
            args[i] = "tmp_"
            call = "%s(%s)" % (name, ", ".join(args))
            body = "%s tmp_ = %s; " % (t, pn)
            if ret == "void":
                body += "%s; %s = tmp_;" % (call, pn)
            else:
                body += "%s r_ = %s; %s = tmp_; return r_;" % (ret, call, pn)
            extra.append((m.end(), "template<class T_, int N_, int... I_> inline %s %s(%s) { %s }" % (ret, name, ", ".join(sig), body)))
    # insert each overload after the end of its function
    for pos, code in sorted(extra, reverse=True):
        depth, j = 1, pos
        while depth and j < len(text):
            depth += {"{": 1, "}": -1}.get(text[j], 0)
            j += 1
        text = text[:j] + "\n" + code + "\n" + text[j:]
    return text


def block_struct(name, body):
    members = []
    decls = []
    for d in [d.strip() for d in body.split(";") if d.strip()]:
        m = re.match(r"(\w+)\s+(\w+(?:\s*,\s*\w+)+)$", d)   # float a, b, c: one member each
        decls += ["%s %s" % (m.group(1), n.strip()) for n in m.group(2).split(",")] if m else [d]
    for decl in decls:
        m = re.match(r"(\w+)\s+(\w+)\s*(\[[^\]]*\])?$", decl)
        if not m:
            raise RuntimeError("cannot parse block member: " + decl)
        t, n, arr = m.group(1), m.group(2), m.group(3) or ""
        ct = "mat3_std140" if t == "mat3" else t
        al = STD140_ALIGN.get(t)
        if arr and t in ("float", "int", "uint"):
            raise RuntimeError("std140 scalar arrays are not modelled: " + decl)
        members.append("%s%s %s%s;" % ("alignas(%d) " % al if al else "", ct, n, arr))
    return "struct %s { %s };" % (name, " ".join(members))


def translate(module, kernel, moddir):
    src = os.path.join(moddir, module, kernel + ".comp")
    text = cpp(resolve_includes(src, moddir))
    binds = []   # (binding, name, kind, is_array)
    blocks = []  # (kind, instance)

    def uniform_block(m):
        lay, name, body, inst = m.group(1), m.group(2), m.group(3), m.group(4)
        if "push_constant" in lay:
            kind = "push"
        else:
            b = int(re.search(r"binding\s*=\s*(\d+)", lay).group(1))
            kind = "global" if b == 0 else "uniform"
        blocks.append((kind, inst))
        return block_struct(name, body) + " static %s %s;" % (name, inst)

    ls = re.search(r"layout\s*\(\s*local_size_x\s*=\s*(\d+)\s*,\s*local_size_y\s*=\s*(\d+)[^)]*\)\s*in\s*;", text)
    local = (int(ls.group(1)), int(ls.group(2))) if ls else (8, 8)
    text = re.sub(r"layout\s*\(([^)]*)\)\s*in\s*;", "", text)
    text = re.sub(r"layout\s*\(([^)]*)\)\s*uniform\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", uniform_block, text, flags=re.S)

    def resource(m):
        lay, typ, name, arr = m.group(1), m.group(3), m.group(4), m.group(5)
        b = int(re.search(r"binding\s*=\s*(\d+)", lay).group(1))
        binds.append((b, name, typ, bool(arr)))
        t = "res_array<%s>" % typ if arr else typ
        return "static %s %s;" % (t, name)

    text = re.sub(r"layout\s*\(([^)]*)\)\s*uniform\s+((?:writeonly|readonly)\s+)?(sampler2D|usampler2D|image2D|uimage2D)\s+(\w+)\s*(\[\s*\])?\s*;",
                  resource, text, flags=re.S)
    buffers = []   # (binding, instance, member, type)

    def ssbo(m):
        lay, name, typ, member, inst = m.group(1), m.group(2), m.group(3), m.group(4), m.group(5)
        b = int(re.search(r"binding\s*=\s*(\d+)", lay).group(1))
        buffers.append((b, inst, member, typ))
        return "struct %s { %s *%s; }; static %s %s;" % (name, typ, member, name, inst)

    # storage buffers of one unsized array: a pointer bound by the runner
    text = re.sub(r"layout\s*\(([^)]*)\)\s*(?:(?:readonly|writeonly|volatile|coherent)\s+)*buffer\s+(\w+)\s*"
                  r"\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*(\w+)\s*;", ssbo, text)
    if re.search(r"\bbuffer\b", text):
        raise RuntimeError("%s/%s uses buffers other than one unsized array (not modelled)" % (module, kernel))
    # workgroup shared arrays: one copy per emulation thread, which runs one workgroup at a time
    text, nshared = re.subn(r"\bshared\s+(\w+)\s+(\w+)\s*\[([^\]]+)\]\s*;",
                            r"static thread_local shared_arr<\1, (\3)> \2;", text)
    if re.search(r"\bshared\b", text):
        raise RuntimeError("%s/%s: shared declaration not understood" % (module, kernel))
    # parameter qualifiers
    text = re.sub(r"\b(?:inout|out)\s+(const\s+)?(\w+)\s+(\w+)", r"\2 &\3", text)
    text = re.sub(r"\bin\s+(const\s+)?(\w+)\s+(\w+)", r"\2 \3", text)
    text = text.replace("^^", "!=")
    # arrays are passed by value in GLSL: array parameters of function definitions become const
    text = re.sub(r"^(\w+\s+\w+\s*\()([^;{}()]*)(\)\s*\{)",
                  lambda m: m.group(1) + re.sub(r"(?<![&\w])(\w+)\s+(\w+)\s*\[(\d+)\]", r"const \1 \2[\3]", m.group(2)) + m.group(3),
                  text, flags=re.M)
    text = replace_array_ctors(text)
    text = scalar_swizzles(text)
    text = swizzle_overloads(text)
    # float literals are single precision in GLSL
    text = re.sub(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])", r"\1f", text)
    text = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", text)
    nphase, coop = 1, False
    if nshared:
        try:
            text, nphase = phases(text)
        except RuntimeError:
            coop = True   # barrier() inside functions: cooperative invocations (glsl.cpp)
    ident = module.replace("-", "_")
    ns = "sh_%s_%s" % (ident, kernel)
    entry = ["extern \"C\" void ref_%s_%s(const ref_dispatch_t *dp)" % (ident, kernel), "{", "  using namespace %s;" % ns]
    for kind, inst in blocks:
        field = {"push": "push", "uniform": "uniform", "global": "global"}[kind]
        entry.append("  if(dp->%s) memcpy(&%s, dp->%s, sizeof(%s));" % (field, inst, field, inst))
    for b, name, typ, arr in binds:
        if arr:
            entry.append("  for(int e = 0; e < 32; e++) %s[e].im = dp->bind[%d][e];" % (name, b))
        else:
            entry.append("  %s.im = dp->bind[%d][0];" % (name, b))
    for b, inst, member, typ in buffers:
        entry.append("  %s.%s = (%s *)dp->buf[%d];" % (inst, member, typ, b))
    if coop:
        LX, LY = local
        entry += [
            "  // workgroups: the node size over DT_LOCAL_SIZE (graph-run-nodes-record-cmd.h:377-380)",
            "  glsl::run_workgroups_coop((dp->wd + 7) / 8, (dp->ht + 7) / 8, dp->dp, %d, %d, %s::shader_main);" % (LX, LY, ns),
            "}",
        ]
        return ("// generated from %s by oracle/glsl/translate.py\n#include \"glsl.hpp\"\n#include <cstring>\n"
                "namespace %s {\nusing namespace glsl;\n%s\n} // namespace\n%s\n") % (src, ns, text, "\n".join(entry))
    if nshared:
        LX, LY = local
        entry += [
            "  // workgroups: the node size over DT_LOCAL_SIZE (graph-run-nodes-record-cmd.h:377-380)",
            "  const int GX = (dp->wd + 7) / 8, GY = (dp->ht + 7) / 8, D = dp->dp;",
            "#pragma omp parallel for collapse(3) schedule(static)",
            "  for(int z = 0; z < D; z++) for(int wy = 0; wy < GY; wy++) for(int wx = 0; wx < GX; wx++)",
            "    for(int ph = 0; ph < %d; ph++)" % nphase,
            "      for(int ly = 0; ly < %d; ly++) for(int lx = 0; lx < %d; lx++)" % (LY, LX),
            "      {",
            "        glsl::gl_GlobalInvocationID = glsl::uvec3((glsl::uint)(wx * %d + lx), (glsl::uint)(wy * %d + ly), (glsl::uint)z);" % (LX, LY),
            "        glsl::gl_LocalInvocationID = glsl::uvec3((glsl::uint)lx, (glsl::uint)ly, 0u);",
            "        glsl::gl_WorkGroupID = glsl::uvec3((glsl::uint)wx, (glsl::uint)wy, (glsl::uint)z);",
            "        glsl::gl_LocalInvocationIndex = (glsl::uint)(ly * %d + lx);" % LX,
            "        glsl::glsl_phase_ = ph;",
            "        shader_main();",
            "      }",
            "}",
        ]
        return ("// generated from %s by oracle/glsl/translate.py\n#include \"glsl.hpp\"\n#include <cstring>\n"
                "namespace %s {\nusing namespace glsl;\n%s\n} // namespace\n%s\n") % (src, ns, text, "\n".join(entry))
    entry += [
        "  const int W = (dp->wd + 7) / 8 * 8, H = (dp->ht + 7) / 8 * 8, D = dp->dp;",
        "#pragma omp parallel for collapse(2) schedule(static)",
        "  for(int z = 0; z < D; z++) for(int y = 0; y < H; y++)",
        "    for(int x = 0; x < W; x++)",
        "    {",
        "      glsl::gl_GlobalInvocationID = glsl::uvec3((glsl::uint)x, (glsl::uint)y, (glsl::uint)z);",
        "      glsl::gl_LocalInvocationID = glsl::uvec3((glsl::uint)(x % 8), (glsl::uint)(y % 8), 0u);",
        "      glsl::gl_WorkGroupID = glsl::uvec3((glsl::uint)(x / 8), (glsl::uint)(y / 8), (glsl::uint)z);",
        "      glsl::gl_LocalInvocationIndex = (glsl::uint)((y % 8) * 8 + x % 8);",
        "      shader_main();",
        "    }",
        "}",
    ]
    tu = ("// generated from %s by oracle/glsl/translate.py\n#include \"glsl.hpp\"\n#include <cstring>\n"
          "namespace %s {\nusing namespace glsl;\n%s\n} // namespace\n%s\n") % (src, ns, text, "\n".join(entry))
    return tu


def phases(text):
    """Barriers: a shader whose main body is a prefix of statements followed by
    compound statements separated by barrier() runs as phases. Every
    invocation of a workgroup runs phase k before any runs phase k+1; the
    prefix (invocation ids, an early return) runs in every phase and the k-th
    top level block only in phase k. Returns (text, number of phases)."""
    m = re.search(r"void shader_main\(\)\s*\{", text)
    i = m.end()
    out = [text[:i], " glsl_bar_ = 0;"]
    depth, j, nbar, seen_block = 1, i, 0, False
    while depth:
        c = text[j]
        if depth == 1 and text.startswith("barrier();", j):
            out.append("glsl_bar_++;")
            nbar += 1
            j += len("barrier();")
            continue
        if c == "{":
            if depth == 1:
                prev = text[:j].rstrip()[-1]
                if prev not in ";{}":
                    raise RuntimeError("a top level statement other than a block after the prefix")
                out.append("if(glsl_bar_ == glsl_phase_) ")
                seen_block = True
            depth += 1
        elif c == "}":
            depth -= 1
        elif depth == 1 and seen_block and not c.isspace():
            raise RuntimeError("statements between the barrier phases are not modelled")
        out.append(c)
        j += 1
    out.append(text[j:])
    if re.search(r"\bbarrier\s*\(", "".join(out)):
        raise RuntimeError("barrier() below the top level of main is not modelled")
    return "".join(out), nbar + 1


def gen_swizzles():
    """glsl_swizzle.inc: the swizzle members of 2, 3 and 4 component vectors."""
    sets = ["xyzw", "rgba"]
    lines = []
    for n in (2, 3, 4):
        mem = []
        for s in sets:
            letters = s[:n]
            import itertools
            for m in (2, 3, 4):
                for combo in itertools.product(range(n), repeat=m):
                    name = "".join(letters[i] for i in combo)
                    mem.append("swz<T, %d, %s> %s;" % (n, ", ".join(str(i) for i in combo), name))
        lines.append("#define GLSL_SWIZZLES_%d %s" % (n, " ".join(mem)))
    return "\n".join(lines) + "\n"


def build(moddir=DEFAULT_MODULES, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    open(os.path.join(OUT, "glsl_swizzle.inc"), "w").write(gen_swizzles())
    srcs = []
    for mod, k in SHADERS:
        tu = translate(mod, k, moddir)
        p = os.path.join(OUT, "%s_%s.cpp" % (mod, k))
        if not os.path.exists(p) or open(p).read() != tu:
            open(p, "w").write(tu)
        srcs.append(p)
    compile_ref()


def compile_ref():
    """Compile the translation units present in oracle/_ref (also on a machine
    without the vkdt sources, from the files translate() wrote)."""
    srcs = sorted(os.path.join(OUT, f) for f in os.listdir(OUT) if f.endswith(".cpp"))
    srcs.append(os.path.join(HERE, "glsl.cpp"))
    flags = ["-O2", "-fno-strict-aliasing", "-std=c++17", "-fno-operator-names", "-ffp-contract=off", "-fopenmp", "-fPIC", "-w",
             "-I" + HERE, "-I" + OUT]
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(s), os.path.getmtime(os.path.join(HERE, "glsl.hpp"))):
            continue
        procs.append((s, subprocess.Popen(["g++"] + flags + ["-c", s, "-o", o], stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    err = []
    for s, p in procs:
        out = p.communicate()[0].decode()
        if p.returncode != 0:
            err.append("%s:\n%s" % (s, out[:4000]))
    if err:
        raise RuntimeError("reference shader build failed:\n" + "\n".join(err))
    so = os.path.join(OUT, "libvkdt_ref.so")
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-o", so] + objs, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError(r.stdout.decode())
    return so


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_MODULES)
    print(os.path.join(OUT, "libvkdt_ref.so"))
