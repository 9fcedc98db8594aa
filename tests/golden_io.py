"""Loading of the golden fixtures (tests/golden/*.npz) and helpers to compare
correlator outputs.  Test infrastructure."""
import ast
import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["c1_plain", "multi", "onebit", "pulsar", "reduced", "reduced_mask", "phase_centers", "phased"]


class Golden:
    def __init__(self, name):
        self.name = name
        self.z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=True)
        self.meta = ast.literal_eval(str(self.z["meta"]))
        self.dels = [bytes(np.asarray(d, dtype=np.uint8)) for d in self.z["del_bytes"]]
        self.nstreams = len(self.meta["streams"])
        self.nint = int(self.meta["n_integrations"])

    def blocks(self, k):
        m = self.meta
        chan = np.asarray(self.z["chan_%d" % k], dtype=np.uint8)
        bb = m["block_bytes"]
        s = m["streams"][k]
        bits, sr = s[7], s[2]
        tps = int(round(512e6 / sr))
        spb_block = bb * 8 // bits
        inv = {}
        key = "%d,%s" % (s[0], s[6])
        for (b, begin, n) in m["invalid"].get(key, []):
            inv.setdefault(b, []).append((begin, n))
        nb = len(chan) // bb
        return [(m["rec0"] + b * spb_block * tps, chan[b * bb:(b + 1) * bb].tobytes(), inv.get(b, []))
                for b in range(nb)]

    def delays(self, k, it):
        return [tuple(int(x) for x in row) for row in self.z["delays_%d_%d" % (k, it)]]

    def slices(self, k):
        m = self.meta
        tint = int(round(m["integration_time_us"] * 512))
        out = []
        for it in range(self.nint):
            s0 = m["start_ticks"] + it * tint
            out.append((s0, s0 + tint, m["slice_samples"], self.delays(k, it)))
        return out

    def protocol_ok(self, k, it, data):
        sha = bytes(np.asarray(self.z["proto_sha_%d_%d" % (k, it)], dtype=np.uint8))
        return hashlib.sha256(data).digest() == sha and len(data) == int(self.z["proto_len_%d_%d" % (k, it)])

    def job(self, protocol_fn):
        """Job dict with protocols regenerated by protocol_fn and checked by digest."""
        m = self.meta
        job = {k: v for k, v in m.items()}
        job["del_bytes"] = self.dels
        for key in ("mask", "lag_window"):  # Mask_parameters of the spectral-reduction cases
            if key in self.z.files:
                job[key] = np.asarray(self.z[key], dtype=np.float32)
        if "uvw" in self.z.files:  # UVW header values [integration][stream][centre][3]
            job["uvw"] = np.asarray(self.z["uvw"], dtype=np.float64)
        protos = []
        for k in range(self.nstreams):
            s = m["streams"][k]
            pr = protocol_fn(self.blocks(k), self.slices(k), s[2], s[7], m["integration_time_us"])
            for it in range(self.nint):
                assert self.protocol_ok(k, it, pr[it]), "protocol of stream %d integration %d differs" % (k, it)
            protos.append(pr)
        job["protocols"] = protos
        return job

    def unpacked_sha(self, k, it):
        return bytes(np.asarray(self.z["unpacked_sha_%d_%d" % (k, it)], dtype=np.uint8))

    @property
    def cor(self):
        return bytes(np.asarray(self.z["cor"], dtype=np.uint8))

    @property
    def tsys(self):
        return bytes(np.asarray(self.z["tsys"], dtype=np.uint8))

    @property
    def stats(self):
        return bytes(np.asarray(self.z["stats"], dtype=np.uint8)).decode()


def phasecal_cases():
    """Phase-cal extraction cases over the channel blocks of scenario fixtures:
    (fixture, stream, integration ticks, first block, extra invalid runs per
    block).  The runs include one that begins where the previous one ends (the
    reference never skips it), runs reaching or passing the block end, a run
    past the end and a run covering a whole block."""
    return {
        "c1_every_third": ("c1_plain", 0, 6144000, 1,
                           {2: [(100, 50), (150, 20), (400, 10)], 3: [(0, 10)], 4: [(31990, 10)],
                            6: [(5, 7), (20, 30)]}),
        "c1_every_block": ("c1_plain", 1, 2048000, 0, {5: [(1000, 3000), (4000, 8)], 8: [(31000, 5000)]}),
        "onebit": ("onebit", 1, 1536000, 0, {3: [(100, 50), (150, 20)], 7: [(0, 4000)], 9: [(3999, 1)]}),
        "multi_scenario_runs": ("multi", 0, 256000, 0, {20: [(1999, 1)], 21: [(2500, 4)]}),
        "multi_short": ("multi", 2, 192000, 2, {4: [(0, 1), (1, 1), (2, 1)], 11: [(600, 2000)]}),
    }


def phasecal_blocks(g, k, first, inject):
    """A fixture's channel blocks from block `first` on, with extra invalid runs."""
    return [(st, d, sorted(list(inv) + [tuple(r) for r in inject.get(b, [])]))
            for b, (st, d, inv) in enumerate(g.blocks(k)) if b >= first]


def parse_cor(data, nchan):
    """Split correlator output bytes into header bytes and visibility arrays.

    Returns (headers: bytes, vis: list of complex64 arrays, one per baseline
    and slice, in file order)."""
    hdr = bytearray()
    vis = []
    p = 0
    while p < len(data):
        hdr += data[p:p + 4]  # file index
        p += 4
        ts = np.frombuffer(data[p:p + 16], dtype=np.int32)
        hdr += data[p:p + 16]
        p += 16
        nbl, nuvw, nstat = int(ts[1]), int(ts[2]), int(ts[3])
        n = nuvw * 32 + nstat * 24
        hdr += data[p:p + n]
        p += n
        for _ in range(nbl):
            hdr += data[p:p + 8]
            p += 8
            vis.append(np.frombuffer(data[p:p + (nchan + 1) * 8], dtype=np.complex64).copy())
            p += (nchan + 1) * 8
    return bytes(hdr), vis


def rel_err(a, b):
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def compare_cor(got, want, nchan, tol):
    """Headers byte-identical; every visibility vector within relative L2 `tol`."""
    hg, vg = parse_cor(got, nchan)
    hw, vw = parse_cor(want, nchan)
    assert hg == hw, "output headers differ"
    assert len(vg) == len(vw)
    worst = max(rel_err(a, b) for a, b in zip(vg, vw))
    assert worst <= tol, "visibility error %.3g exceeds %.3g" % (worst, tol)
    return worst
