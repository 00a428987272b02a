// Malformed residual and ortho pyramid files for the host readers: copies of valid
// .dat files with random bytes changed or the file cut short are opened and every
// tile of the header's range is read; the readers must answer each call with a
// result or an error code, never read or write out of bounds.  Raw deflate streams
// cut from the files and damaged go to tp_inflate_zlib the same way.  Built with
// AddressSanitizer + UndefinedBehaviorSanitizer by tests/test_host_sanitizers.py.
//   dat_fuzz <residual .dat> <ortho .dat> <scratch file> <iterations>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "proland_gb300.h"

namespace {

int g_res_ok = 0, g_orth_ok = 0, g_inflated = 0;  // calls that decoded something

std::vector<uint8_t> read_file(const char *path)
{
    std::vector<uint8_t> b;
    FILE *f = std::fopen(path, "rb");
    if (!f) return b;
    int c;
    while ((c = std::fgetc(f)) != EOF) b.push_back((uint8_t)c);
    std::fclose(f);
    return b;
}

bool write_file(const char *path, const std::vector<uint8_t> &b, size_t n)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(b.data(), 1, n, f) == n;
    std::fclose(f);
    return ok;
}

// a damaged copy: a few bytes changed (the header's 7 fields too, now and then), or
// the file cut short
size_t mutate(std::vector<uint8_t> &b, std::mt19937 &rng)
{
    size_t n = b.size();
    const unsigned kind = rng() % 4;
    if (kind == 0) {
        n = 1 + rng() % (b.size() - 1);
    } else {
        const int flips = 1 + (int)(rng() % 8);
        for (int k = 0; k < flips; ++k) {
            const size_t at = kind == 1 ? rng() % std::min<size_t>(b.size(), 64) : rng() % b.size();
            b[at] = (uint8_t)rng();
        }
    }
    return n;
}

void read_residuals(const char *path)
{
    tp_dat *d = nullptr;
    if (tp_dat_open(path, &d) != TP_OK) return;
    int info[7];
    float scale = 0.0f;
    if (tp_dat_info(d, info, &scale) == TP_OK) {
        std::vector<int16_t> tile(512 * 512);
        int w = 0;
        for (int level = 0; level <= 6; ++level)
            for (int tx = 0; tx < (1 << level) && tx < 8; ++tx)
                for (int ty = 0; ty < (1 << level) && ty < 8; ++ty)
                    g_res_ok += tp_dat_read_tile(d, level, tx, ty, tile.data(), (int)tile.size(), &w) == TP_OK;
    }
    tp_dat_close(d);
}

void read_orthos(const char *path)
{
    tp_ortho_dat *d = nullptr;
    if (tp_ortho_dat_open(path, &d) != TP_OK) return;
    std::vector<uint8_t> tile(4 * 256 * 256);
    std::vector<uint32_t> rgba(256 * 256);
    int w = 0;
    for (int level = 0; level <= 5; ++level)
        for (int tx = 0; tx < (1 << level) && tx < 6; ++tx)
            for (int ty = 0; ty < (1 << level) && ty < 6; ++ty) {
                g_orth_ok += tp_ortho_dat_read_tile(d, level, tx, ty, tile.data(), (int)tile.size(), &w) == TP_OK;
                tp_ortho_dat_read_rgba(d, level, tx, ty, rgba.data(), (int)rgba.size(), &w);
            }
    tp_ortho_dat_close(d);
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 5) {
        std::printf("usage: %s residual.dat ortho.dat scratch iterations\n", argv[0]);
        return 2;
    }
    const std::vector<uint8_t> res = read_file(argv[1]), orth = read_file(argv[2]);
    if (res.size() < 64 || orth.size() < 64) {
        std::printf("cannot read the inputs\n");
        return 2;
    }
    const int iters = std::atoi(argv[4]);
    std::mt19937 rng(7);
    for (int it = 0; it < iters; ++it) {
        std::vector<uint8_t> b = (it & 1) ? orth : res;
        const size_t n = mutate(b, rng);
        if (!write_file(argv[3], b, n)) return 3;
        if (it & 1)
            read_orthos(argv[3]);
        else
            read_residuals(argv[3]);
        // a stretch of the file behind a valid zlib header (so that the decoder gets to
        // the block headers and code tables), damaged and cut at random
        std::vector<uint8_t> out(1 << 18);
        const size_t from = rng() % res.size(), len = 1 + rng() % 4096;
        std::vector<uint8_t> z = {0x78, 0x9C};
        z.insert(z.end(), res.begin() + (long)from, res.begin() + (long)std::min(res.size(), from + len));
        for (int k = 0; k < 3; ++k) z[2 + rng() % (z.size() - 2)] = (uint8_t)rng();
        size_t written = 0;
        g_inflated += tp_inflate_zlib(z.data(), z.size(), out.data(), out.size(), &written) == TP_OK;
        if (written > out.size()) {
            std::printf("FAIL inflate wrote %zu bytes into %zu\n", written, out.size());
            return 1;
        }
    }
    // the damaged files still decode many tiles: the readers get past the header checks
    std::printf("dat fuzz ok: %d residual tiles, %d ortho tiles, %d streams decoded\n", g_res_ok, g_orth_ok,
                g_inflated);
    return 0;
}
