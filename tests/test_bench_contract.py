"""bench.py's JSON line carries every key of the measurement contract (a
static check of the dict literal it prints: the GPU run is the only place
the line is produced)."""
import ast
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

REQUIRED = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "gpu_launches", "e2e", "roofline", "cpu_baseline", "clocks"}


def _dict_keys(node):
    return {k.value for k in node.keys if isinstance(k, ast.Constant) and isinstance(k.value, str)}


def test_bench_line_keys():
    tree = ast.parse(open(os.path.join(ROOT, "bench.py")).read())
    lines = [n for n in ast.walk(tree) if isinstance(n, ast.Assign) and len(n.targets) == 1 and
             isinstance(n.targets[0], ast.Name) and n.targets[0].id == "line" and isinstance(n.value, ast.Dict)]
    assert lines, "bench.py builds no `line = {...}` dict"
    keys = _dict_keys(lines[-1].value)
    assert REQUIRED <= keys, REQUIRED - keys
    roof = [v for k, v in zip(lines[-1].value.keys, lines[-1].value.values)
            if isinstance(k, ast.Constant) and k.value == "roofline"]
    assert roof and isinstance(roof[0], ast.Name)


def test_roofline_keys():
    tree = ast.parse(open(os.path.join(ROOT, "bench.py")).read())
    roofs = [n for n in ast.walk(tree) if isinstance(n, ast.Assign) and len(n.targets) == 1 and
             isinstance(n.targets[0], ast.Name) and n.targets[0].id == "roof" and isinstance(n.value, ast.Dict)]
    assert roofs
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= _dict_keys(roofs[-1].value)
