// The alpha codebook builders of tx_device.cuh (make_book5, make_book7), run
// on the host: against the books' definition by sorting the 8 codes on
// (value, index) and merging equal values (alpha.rs:79-117's first minimum),
// and against the reference's first-minimum search itself.
#include "tx_device.cuh"

#include <algorithm>
#include <cstdio>
#include <random>

using tx::AlphaBook;

static AlphaBook sorted_book(const uint32_t (&codes)[8]) {
    uint32_t k[8];
    for (int j = 0; j < 8; ++j) k[j] = (codes[j] << 3) | (uint32_t)j;
    std::sort(k, k + 8);
    for (int j = 1; j < 8; ++j)
        if ((k[j] ^ k[j - 1]) < 8u) k[j] = k[j - 1];
    AlphaBook b;
    for (int j = 0; j < 7; ++j) {
        const uint32_t a = k[j] >> 3, c = k[j + 1] >> 3;
        const uint32_t T = std::min((a + c + 2u - ((k[j + 1] & 7u) < (k[j] & 7u) ? 1u : 0u)) >> 1, 255u);
        b.t[j] = T * 0x01010101u;
    }
    b.idx_lo = b.idx_hi = b.val_lo = b.val_hi = 0;
    for (int j = 0; j < 4; ++j) {
        b.idx_lo |= (k[j] & 7u) << (8 * j);
        b.idx_hi |= (k[j + 4] & 7u) << (8 * j);
        b.val_lo |= (k[j] >> 3) << (8 * j);
        b.val_hi |= (k[j + 4] >> 3) << (8 * j);
    }
    return b;
}

// (index, value) a pixel x gets from a book: the position #{j : x >= T_j}
static void lookup(const AlphaBook &b, uint32_t x, uint32_t &idx, uint32_t &val) {
    int p = 0;
    for (int j = 0; j < 7; ++j) p += x >= (b.t[j] & 0xFFu) ? 1 : 0;
    const uint32_t iw = p < 4 ? b.idx_lo : b.idx_hi, vw = p < 4 ? b.val_lo : b.val_hi;
    idx = (iw >> (8 * (p & 3))) & 0xFFu;
    val = (vw >> (8 * (p & 3))) & 0xFFu;
}

// the reference: the first code of least squared distance
static uint32_t first_min(const uint32_t (&codes)[8], uint32_t x) {
    int least = 1 << 30;
    uint32_t best = 0;
    for (uint32_t j = 0; j < 8; ++j) {
        const int d = ((int)x - (int)codes[j]) * ((int)x - (int)codes[j]);
        if (d < least) { least = d; best = j; }
    }
    return best;
}

int main() {
    std::mt19937 rng(11);
    long books = 0, looked = 0, bad = 0;
    auto check_lookups = [&](const AlphaBook &b, const uint32_t (&c)[8], const char *what) {
        for (uint32_t x = 0; x < 256; ++x) {
            uint32_t idx, val;
            lookup(b, x, idx, val);
            const uint32_t ref = first_min(c, x);
            ++looked;
            if (idx != ref || val != c[ref]) {
                if (++bad < 8) printf("%s: x %u gives index %u value %u, reference %u\n", what, x, idx, val, ref);
            }
        }
    };
    // 7-value books: every (min7, max7), min5/max5 on and between the interpolants
    for (int lo7 = 0; lo7 < 256; ++lo7)
        for (int hi7 = lo7; hi7 < 256; ++hi7) {
            int min7 = lo7, max7 = hi7;
            tx::fix_range(min7, max7, 7);
            uint32_t c[8];
            for (int i = 1; i < 7; ++i) c[1 + i] = (uint32_t)(((7 - i) * min7 + i * max7) / 7);
            for (int t = 0; t < 24; ++t) {
                int min5, max5;
                if (t < 6) { min5 = (int)c[2 + t]; max5 = std::min(255, min5 + 5 + (int)(rng() % 60)); }
                else if (t < 12) { max5 = (int)c[2 + (t - 6)]; min5 = std::max(0, max5 - 5 - (int)(rng() % 60)); }
                else { min5 = (int)(rng() % 256); max5 = (int)(rng() % 256); if (min5 > max5) std::swap(min5, max5); }
                tx::fix_range(min5, max5, 5);
                c[0] = (uint32_t)min5;
                c[1] = (uint32_t)max5;
                const AlphaBook f = tx::make_book7((uint32_t)min5, (uint32_t)max5, c), g = sorted_book(c);
                bool same = f.idx_lo == g.idx_lo && f.idx_hi == g.idx_hi && f.val_lo == g.val_lo && f.val_hi == g.val_hi;
                for (int j = 0; j < 7; ++j) same = same && f.t[j] == g.t[j];
                ++books;
                if (!same && ++bad < 8) printf("book7 min7 %d max7 %d min5 %d max5 %d differs\n", min7, max7, min5, max5);
                if (books % 41 == 0) check_lookups(f, c, "book7");
            }
        }
    // 5-value books: every (min5, max5)
    for (int lo = 0; lo < 256; ++lo)
        for (int hi = lo; hi < 256; ++hi) {
            int min5 = lo, max5 = hi;
            tx::fix_range(min5, max5, 5);
            uint32_t c[8];
            c[0] = (uint32_t)min5;
            c[1] = (uint32_t)max5;
            for (int i = 1; i < 5; ++i) c[1 + i] = (uint32_t)(((5 - i) * min5 + i * max5) / 5);
            c[6] = 0;
            c[7] = 255;
            const AlphaBook f = tx::make_book5((uint32_t)min5, (uint32_t)max5, c);
            ++books;
            check_lookups(f, c, "book5");
        }
    printf("books %ld, pixel lookups %ld, mismatches %ld\n", books, looked, bad);
    return bad ? 1 : 0;
}
