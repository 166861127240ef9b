// Result images, in place of the reference's MATLAB viewers
// (tomography/convert_to_tiff.m, tomography/projections_sino_tiff.m): every
// slice of the reconstructions, or every projection and sinogram, written as
// one TIFF file.
//
//   to_tiff [fbp|sub|sino]    ($ROOT_CT_DIR, $EXP_CT_NAME as the drivers)
//
// fbp  (convert_to_tiff.m:31-63): slice j of fbp{k}.dat and fbp_tv{k}.dat ->
//      $ROOT_CT_DIR/$EXP_CT_NAME/fbp_images/fbp{j}.tiff and
//      fbp_tv_images/fbp_tv{j}.tiff, (nimage+add)^2 pixels each;
// sub  (convert_sub_to_tiff.m:31-64): the same for the sub-sampled results
//      fbp_sub{k}.dat and fbp_sub_tv{k}.dat -> fbp_sub_images/,
//      fbp_sub_tv_images/; the image side is the one tv_hpc writes with
//      Sub_Sample_Radial = nsub, floor((nimage+add-1)/nsub)+1 (the MATLAB
//      script reads (nimage+add)^2, right only for nsub = 1);
// sino (projections_sino_tiff.m:34-63): projection j of projections{k}.dat ->
//      projections_images/projections{j}.tiff (nimage^2) and slice j of
//      sinograms{k}.dat -> sinogram_images/sinogram{j}.tiff
//      ((nimage+add) x nfiles).
//
// Pixels are what MATLAB's imwrite writes for a double matrix: 8-bit grey,
// round(255 v) with v clipped to [0, 1].  ACUMEN_TIFF=float writes the
// 32-bit floats themselves instead (lossless).  MATLAB's reshape makes the
// file's fastest index (x, or the detector bin) the image row, so image row r,
// column c holds element (x = r, y = c); the files keep that orientation.
//
// The slice-to-file split is the one the drivers write with (the reference's
// single-precision ceiling/floor of k / (count / nfiles)).  convert_to_tiff.m
// locates the fbp files with the sinogram count (rtmp2) and the fbp offsets
// with the reconstruction count (rtmp); it is only consistent when the two
// counts agree, so here both use n_files_rec, as fbp_hpc and tv_hpc write.
#include <sys/stat.h>

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>

#include "hpc_io.h"

using namespace hpc;

namespace {

void put16(std::vector<uint8_t>& b, uint16_t v)
{
    b.push_back(v & 0xff);
    b.push_back(v >> 8);
}
void put32(std::vector<uint8_t>& b, uint32_t v)
{
    for (int i = 0; i < 4; ++i) b.push_back((v >> (8 * i)) & 0xff);
}

// Baseline little-endian TIFF, one strip: `rows` x `cols` pixels with pixel
// (r, c) = data[c * rows + r] (the column-major matrix MATLAB writes).
void write_tiff(const std::string& path, const float* data, int rows, int cols, bool as_float)
{
    const uint32_t bps = as_float ? 32 : 8;
    const unsigned long long total = (unsigned long long)rows * (unsigned long long)cols * (bps / 8);
    if (total > 0xFFFF0000ull) throw Fail("image too large for a baseline TIFF: " + path);   // 32-bit offsets
    const uint32_t nbytes = (uint32_t)total;
    std::vector<uint8_t> img;
    img.reserve(nbytes);
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            const float v = data[(size_t)c * rows + r];
            if (as_float) {
                uint32_t u;
                std::memcpy(&u, &v, 4);
                put32(img, u);
            } else {
                const float cl = v > 1.f ? 1.f : (v > 0.f ? v : 0.f);   // NaN -> 0
                img.push_back((uint8_t)std::lround(255.0 * (double)cl));
            }
        }
    // header (8) + pixels + IFD (2 + 12 n + 4) + two resolution rationals
    const int ntags = as_float ? 12 : 11;
    const uint32_t ifd = 8 + nbytes + (nbytes & 1);
    const uint32_t res = ifd + 2 + 12 * ntags + 4;
    std::vector<uint8_t> b;
    b.push_back('I');
    b.push_back('I');
    put16(b, 42);
    put32(b, ifd);
    b.insert(b.end(), img.begin(), img.end());
    if (nbytes & 1) b.push_back(0);
    put16(b, (uint16_t)ntags);
    auto tag = [&](uint16_t id, uint16_t type, uint32_t count, uint32_t value) {
        put16(b, id);
        put16(b, type);
        put32(b, count);
        if (type == 3 && count == 1) {   // SHORT: left-justified in the value field
            put16(b, (uint16_t)value);
            put16(b, 0);
        } else {
            put32(b, value);
        }
    };
    tag(256, 4, 1, (uint32_t)cols);   // ImageWidth
    tag(257, 4, 1, (uint32_t)rows);   // ImageLength
    tag(258, 3, 1, bps);              // BitsPerSample
    tag(259, 3, 1, 1);                // Compression: none
    tag(262, 3, 1, 1);                // PhotometricInterpretation: BlackIsZero
    tag(273, 4, 1, 8);                // StripOffsets
    tag(277, 3, 1, 1);                // SamplesPerPixel
    tag(278, 4, 1, (uint32_t)rows);   // RowsPerStrip
    tag(279, 4, 1, nbytes);           // StripByteCounts
    tag(282, 5, 1, res);              // XResolution
    tag(283, 5, 1, res + 8);          // YResolution
    if (as_float) tag(339, 3, 1, 3);  // SampleFormat: IEEE float
    put32(b, 0);                      // no next IFD
    for (int i = 0; i < 2; ++i) {     // 72 / 1 pixels per inch
        put32(b, 72);
        put32(b, 1);
    }
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Fail("cannot write " + path);
    const size_t w = std::fwrite(b.data(), 1, b.size(), f);
    std::fclose(f);
    if (w != b.size()) throw Fail("short write to " + path);
}

bool exists(const std::string& p)
{
    struct stat st;
    return ::stat(p.c_str(), &st) == 0;
}

void make_dir(const std::string& p)
{
    if (::mkdir(p.c_str(), 0755) != 0 && errno != EEXIST) throw Fail("cannot create " + p);
}

// Item k (1-based) of `count` items split over `nf` files, `per` floats each.
bool read_item(const std::string& dir, const std::string& base, int k, int count, int nf, size_t per,
               std::vector<float>& out)
{
    const Where w = locate(k, count, nf);
    const std::string path = dir + fnum(base, w.file);
    if (!exists(path)) return false;
    out.resize(per);
    File f(path, false);
    f.read(w.item * (long long)per, out.data(), per);
    return true;
}

}  // namespace

int main(int argc, char** argv)
{
    try {
        const std::string mode = argc > 1 ? argv[1] : "fbp";
        if (mode != "fbp" && mode != "sub" && mode != "sino") throw Fail("usage: to_tiff [fbp|sub|sino]");
        const bool as_float = env("ACUMEN_TIFF", false) == "float";
        const std::string rec = recon_dir();
        const std::string wdir = env("ROOT_CT_DIR") + "/" + env("EXP_CT_NAME") + "/";
        const FileInfo fi = read_fileinfo(rec);
        const int add = fi.nimage % 2 == 0 ? 1 : 0;
        const int n = fi.nimage + add;
        std::vector<float> buf;
        int written = 0;
        if (mode == "fbp" || mode == "sub") {
            const bool sub = mode == "sub";
            const std::string ns = env("Sub_Sample_Radial", false);
            const int nsub = sub && !ns.empty() ? std::atoi(ns.c_str()) : 1;
            if (nsub < 1) throw Fail("Sub_Sample_Radial must be >= 1");
            const int side = (int)std::floor((float)(n - 1) / (float)nsub) + 1;
            for (const std::string base : {sub ? "fbp_sub" : "fbp", sub ? "fbp_sub_tv" : "fbp_tv"}) {
                if (!exists(rec + fnum(base, 1))) {
                    std::cout << "no " << base << "1.dat: skipped\n";
                    continue;
                }
                const std::string out = wdir + base + "_images/";
                make_dir(out);
                for (int j = 1; j <= fi.nimage; ++j) {
                    if (!read_item(rec, base, j, fi.nimage, fi.n_files_rec, (size_t)side * side, buf))
                        throw Fail("missing file for " + base + " slice " + std::to_string(j));
                    write_tiff(out + base + std::to_string(j) + ".tiff", buf.data(), side, side, as_float);
                    ++written;
                }
            }
        } else {
            const std::string outp = wdir + "projections_images/", outs = wdir + "sinogram_images/";
            make_dir(outp);
            make_dir(outs);
            for (int j = 1; j <= fi.nfiles; ++j) {
                if (!read_item(rec, "projections", j, fi.nfiles, fi.n_files_sino,
                               (size_t)fi.nimage * fi.nimage, buf))
                    throw Fail("missing file for projection " + std::to_string(j));
                write_tiff(outp + "projections" + std::to_string(j) + ".tiff", buf.data(), fi.nimage, fi.nimage,
                           as_float);
                ++written;
            }
            for (int j = 1; j <= fi.nimage; ++j) {
                if (!read_item(rec, "sinograms", j, fi.nimage, fi.n_files_sino, (size_t)n * fi.nfiles, buf))
                    throw Fail("missing file for sinogram " + std::to_string(j));
                write_tiff(outs + "sinogram" + std::to_string(j) + ".tiff", buf.data(), n, fi.nfiles, as_float);
                ++written;
            }
        }
        std::cout << "to_tiff: " << written << " images\n";
        return 0;
    } catch (const std::exception& e) {
        std::cerr << "to_tiff: " << e.what() << "\n";
        return 1;
    }
}
