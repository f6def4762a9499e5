// Host check of the tar header rules the rescued output's tar walk runs on the GPU
// (gpuzip_gb300/csrc/gi_tar.h), used by tests/test_tar_rules.py: reads 12-byte number fields from
// the file argv[1] and 512-byte headers from argv[2], and prints for each field "<ok> <value>"
// and for each header "<valid>", one per line.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "gi_tar.h"

static std::vector<uint8_t> slurp(const char* path) {
    std::vector<uint8_t> v;
    FILE* f = fopen(path, "rb");
    if (!f) return v;
    uint8_t buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) v.insert(v.end(), buf, buf + n);
    fclose(f);
    return v;
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    std::vector<uint8_t> fields = slurp(argv[1]), headers = slurp(argv[2]);
    for (size_t i = 0; i + 12 <= fields.size(); i += 12) {
        uint64_t v = 0;
        bool ok = tar_octal(fields.data() + i, 12, v);
        printf("%d %llu\n", ok ? 1 : 0, (unsigned long long)(ok ? v : 0));
    }
    for (size_t i = 0; i + 512 <= headers.size(); i += 512) printf("%d\n", tar_header_valid(headers.data() + i) ? 1 : 0);
    return 0;
}
