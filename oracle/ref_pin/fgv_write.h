/* Writer for the golden-vector container used by the pin harnesses (test infrastructure).
 *
 * File layout ("FGV1"): the 4-byte magic, then records until end of file. A record is
 *   uint32 name_len, name bytes, uint32 ndim, uint64 dims[ndim], float64 data[prod(dims)]
 * all little-endian. tests/golden/fgv.py reads the same layout. */
#ifndef FPDE_FGV_WRITE_H
#define FPDE_FGV_WRITE_H
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include <vector>
#include <string>

struct FgvWriter {
    FILE *f;
    explicit FgvWriter(const char *path) {
        f = fopen(path, "wb");
        if (!f) { perror(path); exit(2); }
        fwrite("FGV1", 1, 4, f);
    }
    ~FgvWriter() { if (f) fclose(f); }
    void put(const std::string &name, const std::vector<uint64_t> &dims, const double *data) {
        uint32_t nl = (uint32_t)name.size();
        fwrite(&nl, 4, 1, f);
        fwrite(name.data(), 1, nl, f);
        uint32_t nd = (uint32_t)dims.size();
        fwrite(&nd, 4, 1, f);
        uint64_t n = 1;
        for (uint64_t d : dims) { fwrite(&d, 8, 1, f); n *= d; }
        if (n) fwrite(data, 8, n, f);
    }
    void put(const std::string &name, const std::vector<double> &v) {
        put(name, {(uint64_t)v.size()}, v.data());
    }
    void scalar(const std::string &name, double v) { put(name, {}, &v); }
};
#endif
