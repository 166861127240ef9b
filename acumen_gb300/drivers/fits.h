// Minimal reader of a FITS primary array (the part of cfitsio that
// tomography/fits_to_hpc.F90 uses: ftgknj for NAXIS1/NAXIS2 and ftgpve for the
// pixel values as single precision).  Follows the FITS standard: 2880-byte
// blocks, 80-character header cards up to END, big-endian data of BITPIX
// 8 (unsigned), 16, 32, 64 (signed integers), -32 or -64 (IEEE floats), and
// physical value = BZERO + BSCALE * stored value.  Byte order is converted
// with shifts, so the code is the same on little- and big-endian hosts.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hpc_io.h"

namespace hpc {

struct FitsImage {
    long naxis1 = 0, naxis2 = 0;   // NAXIS1 is the fastest axis
    std::vector<float> data;       // naxis1 * naxis2 values, NAXIS1 fastest
};

namespace fits_detail {

inline std::string trim(const std::string& s)
{
    size_t a = s.find_first_not_of(' '), b = s.find_last_not_of(' ');
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

inline uint64_t be_bytes(const unsigned char* p, int n)
{
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v = (v << 8) | p[i];
    return v;
}

}  // namespace fits_detail

inline FitsImage read_fits(const std::string& path)
{
    using namespace fits_detail;
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw Fail("cannot open " + path);
    struct Closer {
        FILE* f;
        ~Closer() { std::fclose(f); }
    } closer{f};
    int bitpix = 0, naxis = -1;
    long ax[3] = {0, 0, 0};
    double bzero = 0.0, bscale = 1.0;
    bool end = false, simple = false;
    char block[2880];
    for (int nblk = 0; !end; ++nblk) {
        if (std::fread(block, 1, 2880, f) != 2880) throw Fail(path + ": truncated FITS header");
        for (int c = 0; c < 36 && !end; ++c) {
            const std::string card(block + 80 * c, 80);
            const std::string key = trim(card.substr(0, 8));
            if (key == "END") {
                end = true;
                break;
            }
            if (card.size() < 10 || card[8] != '=') continue;
            std::string val = card.substr(10);
            const size_t slash = val.find('/');
            if (slash != std::string::npos && val.find('\'') == std::string::npos) val = val.substr(0, slash);
            val = trim(val);
            if (key == "SIMPLE") simple = (val == "T");
            else if (key == "BITPIX") bitpix = std::atoi(val.c_str());
            else if (key == "NAXIS") naxis = std::atoi(val.c_str());
            else if (key == "NAXIS1") ax[0] = std::atol(val.c_str());
            else if (key == "NAXIS2") ax[1] = std::atol(val.c_str());
            else if (key == "NAXIS3") ax[2] = std::atol(val.c_str());
            else if (key == "BZERO") bzero = std::atof(val.c_str());
            else if (key == "BSCALE") bscale = std::atof(val.c_str());
        }
        if (nblk > 1000) throw Fail(path + ": no END card");
    }
    if (!simple) throw Fail(path + ": not a FITS file (SIMPLE = T missing)");
    if (naxis < 2 || ax[0] < 1 || ax[1] < 1 || (naxis > 2 && ax[2] > 1))
        throw Fail(path + ": expected a 2-D primary array");
    const int bytes = std::abs(bitpix) / 8;
    if (!(bitpix == 8 || bitpix == 16 || bitpix == 32 || bitpix == 64 || bitpix == -32 || bitpix == -64))
        throw Fail(path + ": unsupported BITPIX " + std::to_string(bitpix));
    FitsImage img;
    img.naxis1 = ax[0];
    img.naxis2 = ax[1];
    const size_t n = (size_t)ax[0] * (size_t)ax[1];
    std::vector<unsigned char> raw(n * bytes);
    if (std::fread(raw.data(), 1, raw.size(), f) != raw.size()) throw Fail(path + ": truncated FITS data");
    img.data.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const unsigned char* p = raw.data() + i * bytes;
        const uint64_t u = be_bytes(p, bytes);
        double v;
        switch (bitpix) {
        case 8: v = (double)(uint8_t)u; break;
        case 16: v = (double)(int16_t)(uint16_t)u; break;
        case 32: v = (double)(int32_t)(uint32_t)u; break;
        case 64: v = (double)(int64_t)u; break;
        case -32: {
            const uint32_t w = (uint32_t)u;
            float x;
            std::memcpy(&x, &w, 4);
            v = x;
            break;
        }
        default: {
            double x;
            std::memcpy(&x, &u, 8);
            v = x;
        }
        }
        img.data[i] = (float)(bzero + bscale * v);
    }
    return img;
}

}  // namespace hpc
