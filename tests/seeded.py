"""Test restatement of the seeded problem generators: MT19937-64 (Matsumoto &
Nishimura; the engine std::mt19937_64 names) in plain Python, and the draw
order of amr_config_blast / amr_config_kh."""
import math

_M64 = (1 << 64) - 1


class MT64:
    def __init__(self, seed):
        self.mt = [0] * 312
        self.mt[0] = seed & _M64
        for i in range(1, 312):
            self.mt[i] = (6364136223846793005 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 62)) + i) & _M64
        self.idx = 312

    def raw(self):
        if self.idx >= 312:
            mt = self.mt
            for i in range(312):
                x = (mt[i] & 0xFFFFFFFF80000000) | (mt[(i + 1) % 312] & 0x7FFFFFFF)
                xa = x >> 1
                if x & 1:
                    xa ^= 0xB5026F5AA96619E9
                mt[i] = mt[(i + 156) % 312] ^ xa
            self.idx = 0
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000 & _M64
        y ^= (y << 37) & 0xFFF7EEE000000000 & _M64
        y ^= y >> 43
        return y & _M64

    def uniform(self):
        return (self.raw() >> 11) * (1.0 / 9007199254740992.0)


def blast_params(seed, index):
    g = MT64(seed + index)
    s4p = math.sqrt(4.0 * math.pi)
    r0 = 0.05 + 0.10 * g.uniform()
    pin = 5.0 + 45.0 * g.uniform()
    b = (0.5 + 1.5 * g.uniform()) / s4p
    th = 0.5 * math.pi * g.uniform()
    maxlevs = 3 + (g.raw() >> 62)
    return [r0, pin, b, th, 0.5, 0.5], maxlevs


def kh_amplitudes(seed):
    g = MT64(seed)
    out = []
    while len(out) < 16:
        u1, u2 = g.uniform(), g.uniform()
        if u1 <= 0.0:
            u1 = 1.0 / 9007199254740992.0
        r = math.sqrt(-2.0 * math.log(u1))
        out += [r * math.cos(2.0 * math.pi * u2), r * math.sin(2.0 * math.pi * u2)]
    return [1e-3 * a for a in out[:16]]
