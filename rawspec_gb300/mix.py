"""The serving workload: a seeded list of spectrometer jobs with Poisson
arrivals, each a stream of 2-16 RAW blocks with Nchan in {8, 32, 64}, 4- or
8-bit samples of two polarisations and 1-3 products with Nfft in {8, 1024,
65536, 1048576}, Nint in 16..3072 and Npolout in {1, 4, -4}.

Nint is drawn among the values rawspec_initialize accepts for the product
(a divisor or a multiple of the spectra per buffer, rawspec_gpu.cu:587-613),
and the blocks of a job are a whole number of buffers."""
from __future__ import annotations

import numpy as np

NFFTS = (8, 1024, 1 << 16, 1 << 20)
NINTS = (16, 32, 64, 128, 256, 512, 1024, 2048, 3072)


def serving_jobs(n: int = 256, rate: float = 40.0, ntpb: int = 1 << 18, seed: int = 5) -> list[dict]:
    """Jobs in arrival order: dict(arrival [s], Nc, nbits, products [(Nfft, Nint, Npolout)], Nb, blocks)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for _ in range(n):
        t += float(rng.exponential(1.0 / rate))
        nc = int(rng.choice([8, 32, 64]))
        nbits = int(rng.choice([4, 8]))
        nprod = int(rng.integers(1, 4))
        nts = sorted((int(x) for x in rng.choice(NFFTS, size=nprod, replace=False)), reverse=True)
        nb = max(1, nts[0] // ntpb)
        prods = []
        for nt in nts:
            nss = nb * ntpb // nt
            ok = [na for na in NINTS if (na <= nss and nss % na == 0) or (na > nss and na % nss == 0)]
            prods.append((nt, int(rng.choice(ok)), int(rng.choice([1, 4, -4]))))
        nblk = int(rng.integers(2, 17))
        nblk = max(nb, nblk // nb * nb)
        jobs.append(dict(arrival=t, Nc=nc, nbits=nbits, products=prods, Nb=nb, blocks=nblk, ntpb=ntpb))
    return jobs


def block_bytes(job: dict) -> int:
    """Bytes of one host block of the job (packed bytes for 4-bit samples)."""
    per = 1 if job["nbits"] == 4 else 2 * job["nbits"] // 8
    return job["Nc"] * job["ntpb"] * 2 * per
