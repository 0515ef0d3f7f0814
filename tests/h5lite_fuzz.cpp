// Fuzz driver of the library's HDF5 reader (test_particle_gb300/csrc/h5lite.cpp),
// built by tests/test_h5.py with AddressSanitizer and UndefinedBehaviorSanitizer:
// changes one or two bytes outside the raw data of a valid file, then opens,
// describes and reads every dataset of the file.  Any out-of-bounds access or
// undefined behaviour aborts the process.
//   h5lite_fuzz <file> <positions: int64 list> <work file> <iterations> <seed>
#include "h5lite.cpp"

#include <fstream>
#include <iterator>
#include <random>

int main(int argc, char** argv)
{
    if (argc != 6) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    std::vector<uint8_t> base((std::istreambuf_iterator<char>(in)), {});
    std::ifstream pin(argv[2], std::ios::binary);
    std::vector<char> praw((std::istreambuf_iterator<char>(pin)), {});
    std::vector<int64_t> pos(praw.size() / 8);
    memcpy(pos.data(), praw.data(), pos.size() * 8);
    if (base.empty() || pos.empty()) return 2;
    const long iters = atol(argv[4]);
    std::mt19937_64 rng((uint64_t)atol(argv[5]));
    const char* paths[3][2] = {{"/g", "d"}, {"/", "top"}, {"/particles_fields", "particles"}};
    long ok = 0, refused = 0;
    for (long it = 0; it < iters; it++) {
        std::vector<uint8_t> b(base);
        const int nm = 1 + (int)(rng() % 2);
        for (int k = 0; k < nm; k++) {
            const size_t i = (size_t)pos[rng() % pos.size()];
            const int r = (int)(rng() % 100);
            static const uint8_t special[8] = {0, 1, 2, 3, 4, 0xff, 0x7f, 0x80};
            if (r < 40) b[i] = (uint8_t)rng();
            else if (r < 70) b[i] ^= (uint8_t)(1u << (rng() % 8));
            else if (r < 85) b[i] = special[rng() % 8];
            else
                for (size_t j = i; j < std::min(b.size(), i + 8); j++) b[j] = 0xff;
        }
        FILE* f = fopen(argv[3], "wb");
        if (!f) return 2;
        fwrite(b.data(), 1, b.size(), f);
        fclose(f);
        for (auto& p : paths) {
            tph5::File fl;
            tph5::Dataset ds;
            if (!fl.open(argv[3]) || !fl.dataset(p[0], p[1], ds)) {
                refused++;
                continue;
            }
            std::vector<uint64_t> off(ds.dims.size(), 0), cnt(ds.dims.size());
            uint64_t tot = 1;
            for (size_t d = 0; d < ds.dims.size(); d++) {
                cnt[d] = std::min<uint64_t>(ds.dims[d], 4);
                tot *= cnt[d];
            }
            if (tot * ds.type.size > (64u << 20)) {
                refused++;
                continue;
            }
            std::vector<uint8_t> out(std::max<uint64_t>(tot, 1) * ds.type.size);
            try {
                if (!fl.read(ds, off.data(), cnt.data(), out.data())) {
                    refused++;
                    continue;
                }
            } catch (const std::exception&) {  // an allocation for a corrupted extent
                refused++;
                continue;
            }
            ok++;
            if (ds.type.cls == 0 || ds.type.cls == 1) {
                std::vector<double> v(tot);
                tph5::raw_to_double(ds.type, out.data(), tot, v.data());
            }
            if (ds.type.cls == 6)
                for (uint64_t r = 0; r < tot; r++)
                    for (const auto& m : ds.type.members)
                        if (m.type.cls >= 0 && (uint64_t)m.offset + m.type.size <= ds.type.size)
                            (void)tph5::decode(m.type, out.data() + r * ds.type.size + m.offset);
        }
    }
    printf("FUZZ %ld %ld\n", ok, refused);
    return 0;
}
