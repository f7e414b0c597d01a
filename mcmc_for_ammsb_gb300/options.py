"""Option surface of the sampler, mirroring mcmc::Options (options.h:129-315).

Same long names (``--mcmc.K``), short names (``-K``, ``-m``, ``-n``, ``-x``,
``-i``, ``-I``, ``-h``, ``-f``, ``-c``), defaults (options.h:144-202), the
derived defaults applied in Options::Parse (options.h:257-262) and the
integer syntax of parse_size_t (options.cc:5-67: hex ``0x``, octal leading
``0``, suffixes k/m/g).  Unrecognised arguments are kept in ``remains``
(options.h:244-255 allow_unregistered).  GB300-only options live under
``--gb300.*``.
"""
import math

from . import _native

STRATEGIES = {
    "stratified-random-node": _native.STRATIFIED_RANDOM_NODE,
    "stratified-random-node-links": _native.STRATIFIED_RANDOM_NODE_LINKS,
    "stratified-random-node-nonlinks": _native.STRATIFIED_RANDOM_NODE_NONLINKS,
    "random-edge": _native.RANDOM_EDGE,
}
STRATEGY_NAMES = {v: k for k, v in STRATEGIES.items()}


class NumberFormatError(ValueError):
    """mcmc::NumberFormatException (exception.h)."""


def parse_size_t(arg):
    """options.cc:5-67: decimal, 0x hex, leading-0 octal, k/m/g suffixes."""
    s = arg
    base = 10
    if s[:2] in ("0x", "0X"):
        base, s = 16, s[2:]
    elif s[:1] == "0":
        base, s = 8, s[1:]
    n = 0
    i = 0
    while i < len(s):
        ch = s[i]
        if base == 16 and ch in "0123456789abcdefABCDEF":
            n = n * 16 + int(ch, 16)
        elif base <= 10 and ch.isdigit():
            n = n * base + int(ch)
        elif s[i:].lower() in ("g", "gb"):
            n <<= 30
            break
        elif s[i:].lower() in ("m", "mb"):
            n <<= 20
            break
        elif s[i:].lower() in ("k", "kb"):
            n <<= 10
            break
        else:
            raise NumberFormatError("Unknown characters in number: '%s'" % ch)
        if n >= 1 << 64:
            raise NumberFormatError("Overflow in parse_size_t")
        i += 1
    return n


def parse_int(arg, bits=64, signed=False):
    """mcmc::parse<T> (options.h:40-55) for the VALIDATE_SPECIALIZE types."""
    if arg.startswith("-"):
        v = -parse_size_t(arg[1:])
    else:
        v = parse_size_t(arg)
    lo = -(1 << (bits - 1)) if signed else 0
    hi = (1 << (bits - 1)) - 1 if signed else (1 << bits) - 1
    if v < lo or v > hi:
        raise NumberFormatError("number out of range for type")
    return v


# (long name, short, attribute, kind, default)
_SPEC = [
    ("mcmc.alpha", None, "alpha", "float", 0.0),
    ("mcmc.eta0", None, "eta0", "float", 1.0),
    ("mcmc.eta1", None, "eta1", "float", 1.0),
    ("mcmc.epsilon", None, "epsilon", "float", 0.0000001),
    ("mcmc.a", None, "a", "float", 0.0),
    ("mcmc.b", None, "b", "float", 1024.0),
    ("mcmc.c", None, "c", "float", 0.5),
    ("mcmc.K", "K", "K", "size", 300),
    ("mcmc.mini-batch-size", "m", "mini_batch_size", "size", 0),
    ("mcmc.num-node-sample", "n", "num_node_sample", "size", 0),
    ("mcmc.strategy", None, "strategy", "strategy", _native.STRATIFIED_RANDOM_NODE),
    ("mcmc.sampler.max-source", None, "sampler_max_source", "size", 1),
    ("mcmc.max-iteration", "x", "max_iteration", "size", 10000000),
    ("mcmc.interval", "i", "interval", "size", 0),
    ("mcmc.stats", "I", "stats_print_interval", "size", 0),
    ("mcmc.num-updates", None, "num_updates", "size", 1000),
    ("mcmc.held-out-ratio", "h", "held_out_ratio", "double", 0.0),
    ("mcmc.seed", None, "random_seed", "int", 42),
    ("mcmc.convergence", None, "convergence_threshold", "double", 0.000000000001),
    ("mcmc.input.file", "f", "input_filename_", "str", ""),
    ("mcmc.input.class", "c", "input_class_", "str", "relativity"),
    ("mcmc.input.contiguous", None, "input_contiguous_", "switch", False),
    ("mcmc.input.compressed", None, "input_compressed_", "switch", False),
    ("config", None, "config_file", "str", ""),
    # GB300 options
    ("gb300.pi-dtype", None, "pi_dtype", "dtype", _native.PI_F32),
    ("gb300.chain", None, "chain", "int", 0),
    ("gb300.device", None, "device", "int", 0),
    ("gb300.graph", None, "use_graph", "int", 1),
    ("gb300.pipeline", None, "pipeline", "int", 1),
    ("gb300.verbose", None, "verbose", "int", 0),
]
_BY_LONG = {s[0]: s for s in _SPEC}
_BY_SHORT = {s[1]: s for s in _SPEC if s[1]}


def _convert(kind, text):
    if kind == "float" or kind == "double":
        return float(text)
    if kind == "size":
        return parse_int(text, 64, signed=False)
    if kind == "int":
        return parse_int(text, 32, signed=True)
    if kind == "strategy":
        if text not in STRATEGIES:
            raise ValueError("Unknown strategy")  # types.h:35-36
        return STRATEGIES[text]
    if kind == "dtype":
        t = text.lower()
        if t in ("f32", "float32", "fp32", "float"):
            return _native.PI_F32
        if t in ("bf16", "bfloat16"):
            return _native.PI_BF16
        raise ValueError("pi dtype must be f32 or bf16")
    return text


class Options:
    """mcmc::Options.  ``Options(argv)`` parses like Options::Parse."""

    def __init__(self, argv=None, **overrides):
        for long_name, _, attr, _, default in _SPEC:
            setattr(self, attr, default)
        self.remains = []
        if argv:
            self.parse(list(argv))
        for k, v in overrides.items():
            if not any(s[2] == k for s in _SPEC):
                raise AttributeError("unknown option %s" % k)
            setattr(self, k, v)
        self._derive()

    def parse(self, argv):
        i = 0
        seen = set()
        while i < len(argv):
            tok = argv[i]
            spec = None
            value = None
            if tok.startswith("--"):
                name = tok[2:]
                if "=" in name:
                    name, value = name.split("=", 1)
                spec = _BY_LONG.get(name)
            elif tok.startswith("-") and len(tok) >= 2 and not _looks_numeric(tok):
                spec = _BY_SHORT.get(tok[1])
                if spec is not None and len(tok) > 2:
                    value = tok[2:]
            if spec is None:
                self.remains.append(tok)
                i += 1
                continue
            long_name, _, attr, kind, _ = spec
            if kind == "switch":
                setattr(self, attr, True)
                i += 1
                continue
            if value is None:
                if i + 1 >= len(argv):
                    raise ValueError("option '--%s' requires an argument" % long_name)
                value = argv[i + 1]
                i += 1
            if attr in seen:
                raise ValueError("option '--%s' cannot be specified more than once" % long_name)
            seen.add(attr)
            setattr(self, attr, _convert(kind, value))
            i += 1
        if self.config_file:
            self._parse_config(self.config_file, seen)

    def _parse_config(self, path, seen):
        """po::parse_config_file: `name = value` lines, [section] prefixes."""
        section = ""
        with open(path) as f:
            for raw in f:
                line = raw.split("#", 1)[0].strip()
                if not line:
                    continue
                if line.startswith("[") and line.endswith("]"):
                    section = line[1:-1].strip() + "."
                    continue
                if "=" not in line:
                    raise ValueError("invalid config line: %r" % raw)
                k, v = (x.strip() for x in line.split("=", 1))
                spec = _BY_LONG.get(section + k)
                if spec is None:
                    raise ValueError("unrecognised option '%s' in config" % (section + k))
                if spec[2] in seen:  # command line wins (first store wins)
                    continue
                if spec[3] == "switch":
                    setattr(self, spec[2], v.lower() in ("1", "true", "yes", "on"))
                else:
                    setattr(self, spec[2], _convert(spec[3], v))

    def _derive(self):
        # options.h:257-262
        if self.a == 0.0:
            self.a = math.pow(self.b, -self.c)
        if self.alpha == 0.0 and self.K > 0:
            self.alpha = 1.0 / self.K

    def to_native(self):
        o = _native.AmmsbOptions()
        _native.lib().ammsb_options_default(o)
        for _, _, attr, _, _ in _SPEC:
            if hasattr(o, attr):
                setattr(o, attr, getattr(self, attr))
        return o

    def __repr__(self):
        items = ", ".join("%s=%r" % (s[2], getattr(self, s[2])) for s in _SPEC)
        return "Options(%s)" % items


def _looks_numeric(tok):
    try:
        float(tok)
        return True
    except ValueError:
        return False
