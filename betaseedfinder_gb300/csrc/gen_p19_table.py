#!/usr/bin/env python3
"""Generate p19_table.inc: the Stage0.75 monster-gate regression trees as data.

The reference ships the 16-tree ensemble as nested if/else code
(native/src/p19_monster_gate.hpp:81-2027, the native copy of
src/P19MonsterGate.java). The GPU gate walks the same trees from a node table,
so this script parses that header once and writes the thresholds, leaf values
and feature ids verbatim (as C hexadecimal double literals, so no decimal
round trip can change a bit). The generated file is committed; the script is
only rerun when the reference model changes.

Usage: python gen_p19_table.py <path/to/native/src/p19_monster_gate.hpp>
"""
import os
import re
import sys

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "p19_table.inc")

# Feature expressions exactly as they appear in the reference trees. The id is
# the index used by the device and oracle feature evaluators.
FEATURES = [
    ("scout", "scout"),
    ("p.stage0FullY88", "fullY88"),
    ("p.stage0FullY96", "fullY96"),
    ("p.stage0FullY104", "fullY104"),
    ("p.stage0FullY112", "fullY112"),
    ("p.stage0Y88LargestCluster", "y88Largest"),
    ("p.stage0Y88Width", "y88Width"),
    ("p.stage0Y88Depth", "y88Depth"),
    ("p.stage0Y96LargestCluster", "y96Largest"),
    ("p.stage0Y96Width", "y96Width"),
    ("p.stage0Y96Depth", "y96Depth"),
    ("((double) p.stage0FullY88 / (scout + EPSILON))", "fullY88 / (scout + eps)"),
    ("(p.stage0Y88Width + p.stage0Y88Depth + p.stage0Y96Width + p.stage0Y96Depth)", "sum of widths/depths"),
    ("(p.stage0Y96Width * p.stage0Y96Depth)", "y96 bbox area"),
    ("(p.stage0Y88Width * p.stage0Y88Depth)", "y88 bbox area"),
    ("((double) p.stage0Y88LargestCluster / (p.stage0FullY88 + EPSILON))", "y88Largest / (fullY88 + eps)"),
    ("(p.stage0FullY96 + p.stage0FullY104 + p.stage0FullY112)", "fullY96 + fullY104 + fullY112"),
    ("((double) p.stage0Y96LargestCluster / (p.stage0FullY96 + EPSILON))", "y96Largest / (fullY96 + eps)"),
    ("((double) p.stage0FullY104 / (p.stage0FullY96 + EPSILON))", "fullY104 / (fullY96 + eps)"),
    ("((double) p.stage0FullY96 / (p.stage0FullY88 + EPSILON))", "fullY96 / (fullY88 + eps)"),
    ("(p.stage0Y88LargestCluster + p.stage0Y96LargestCluster)", "y88Largest + y96Largest"),
]
FEATURE_ID = {expr: i for i, (expr, _) in enumerate(FEATURES)}

IF_RE = re.compile(r"^if \((.*) <= ([-+0-9.eE]+)\) \{$")
RET_RE = re.compile(r"^return ([-+0-9.eE]+);$")


def parse_trees(text):
    trees = {}
    for m in re.finditer(r"inline double tree(\d+)\(int scout, const MonsterFeatures& p\) \{\n", text):
        idx = int(m.group(1))
        pos = m.end()
        depth = 1
        end = pos
        while depth:
            ch = text[end]
            if ch == "{":
                depth += 1
            elif ch == "}":
                depth -= 1
            end += 1
        body = text[pos:end - 1]
        toks = [ln.strip() for ln in body.splitlines() if ln.strip()]
        trees[idx] = toks
    if sorted(trees) != list(range(16)):
        raise SystemExit("expected tree0..tree15, found %s" % sorted(trees))
    return [trees[i] for i in range(16)]


def build(toks):
    """Return nodes as (feature, value, left, right) with feature -1 for leaves."""
    nodes = []
    pos = 0

    def node():
        nonlocal pos
        t = toks[pos]
        m = RET_RE.match(t)
        if m:
            pos += 1
            nodes.append([-1, float(m.group(1)), -1, -1, m.group(1)])
            return len(nodes) - 1
        m = IF_RE.match(t)
        if not m:
            raise SystemExit("unparsed tree line: %r" % t)
        expr = m.group(1)
        if expr not in FEATURE_ID:
            raise SystemExit("unknown feature expression: %r" % expr)
        me = len(nodes)
        nodes.append([FEATURE_ID[expr], float(m.group(2)), -1, -1, m.group(2)])
        pos += 1
        left = node()
        if toks[pos] != "} else {":
            raise SystemExit("expected else, got %r" % toks[pos])
        pos += 1
        right = node()
        if toks[pos] != "}":
            raise SystemExit("expected }, got %r" % toks[pos])
        pos += 1
        nodes[me][2] = left
        nodes[me][3] = right
        return me

    root = node()
    if pos != len(toks) or root != 0:
        raise SystemExit("trailing tokens in tree")
    return nodes


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: gen_p19_table.py <path/to/native/src/p19_monster_gate.hpp>")
    src = sys.argv[1]
    text = open(src).read()
    m = re.search(r"THRESHOLD = ([0-9.]+);", text)
    threshold = float(m.group(1))
    eps = float(re.search(r"EPSILON = ([0-9.eE+-]+);", text).group(1))
    all_nodes, roots = [], []
    for toks in parse_trees(text):
        nodes = build(toks)
        base = len(all_nodes)
        roots.append(base)
        for f, v, l, r, lit in nodes:
            all_nodes.append((f, v, l + base if l >= 0 else -1, r + base if r >= 0 else -1, lit))
    lines = [
        "/* Generated by gen_p19_table.py from the reference Stage0.75 monster gate",
        " * (native/src/p19_monster_gate.hpp:25-27 constants, :81-2027 trees).",
        " * Node i: feature id (-1 = leaf), threshold or leaf value, left (<=) / right child.",
        " * Values are hexadecimal double literals, bit-identical to the decimal source. */",
        "#define BSF_P19_TREE_COUNT 16",
        "#define BSF_P19_NODE_COUNT %d" % len(all_nodes),
        "#define BSF_P19_FEATURE_COUNT %d" % len(FEATURES),
        "#define BSF_P19_THRESHOLD %s /* %r */" % (threshold.hex(), threshold),
        "#define BSF_P19_EPSILON %s /* %r */" % (eps.hex(), eps),
        "static const short bsf_p19_root[16] = {%s};" % ", ".join(str(r) for r in roots),
    ]
    feats = ", ".join(str(n[0]) for n in all_nodes)
    lefts = ", ".join(str(n[2]) for n in all_nodes)
    rights = ", ".join(str(n[3]) for n in all_nodes)
    vals = ",\n    ".join("%s /* %s */" % (float(n[4]).hex(), n[4]) for n in all_nodes)
    lines.append("static const signed char bsf_p19_feature[BSF_P19_NODE_COUNT] = {%s};" % feats)
    lines.append("static const short bsf_p19_left[BSF_P19_NODE_COUNT] = {%s};" % lefts)
    lines.append("static const short bsf_p19_right[BSF_P19_NODE_COUNT] = {%s};" % rights)
    lines.append("static const double bsf_p19_value[BSF_P19_NODE_COUNT] = {\n    %s};" % vals)
    lines.append("/* Feature ids: */")
    for i, (_, desc) in enumerate(FEATURES):
        lines.append("/*  %2d: %s */" % (i, desc))
    with open(OUT, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print("wrote %s: %d nodes" % (OUT, len(all_nodes)))


if __name__ == "__main__":
    main()
