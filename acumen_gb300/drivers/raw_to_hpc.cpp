// raw_to_hpc: the normalisation half of tomography/fits_to_hpc.F90.  The
// reference reads FITS files through cfitsio and parses the angle from each
// file name (:57-97, :162-190); that host I/O is outside this library, so the
// stacks come as raw native-endian uint16 files under
// $ROOT_CT_DIR/$EXP_CT_NAME/raw/:
//   projections.u16  nproj x nimage x nimage     OB.u16  nflat x nimage x nimage
//   DF.u16           ndark x nimage x nimage     theta.txt  nproj angles (degrees)
//   info.txt         "nproj nimage nflat ndark"
// Flat and dark frames are averaged (:183-210) and every projection is
// log-normalised (:243, or :244 with ACUMEN_NORM_MODE=1) on the GPU; the
// outputs are the reference's theta.dat, projections{k}.dat (split over
// n_files_sino files of at most ~8e9 bytes, :217-248) and the 4-float
// fileinfo_projections.dat (:255-267).
#include <chrono>

#include "hpc_io.h"

static std::vector<uint16_t> read_u16(const std::string& path, size_t n)
{
    std::vector<uint16_t> v(n);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw hpc::Fail("cannot open " + path);
    const size_t got = std::fread(v.data(), sizeof(uint16_t), n, f);
    std::fclose(f);
    if (got != n) throw hpc::Fail("short read from " + path);
    return v;
}

int main()
{
    try {
        using namespace hpc;
        const auto t0 = std::chrono::steady_clock::now();
        const std::string base = env("ROOT_CT_DIR") + "/" + env("EXP_CT_NAME") + "/";
        const std::string raw = base + "raw/", dir = base + "reconstruction/";
        std::ifstream info(raw + "info.txt");
        int nproj = 0, nimage = 0, nflat = 0, ndark = 0;
        info >> nproj >> nimage >> nflat >> ndark;
        if (!info || nproj < 1 || nimage < 2 || nflat < 1)
            throw Fail("malformed " + raw + "info.txt (nproj nimage nflat ndark)");
        std::printf(" Number of raw projections:  %d\n", nproj);
        std::vector<float> theta(nproj);
        std::ifstream tf(raw + "theta.txt");
        for (auto& t : theta) tf >> t;
        if (!tf) throw Fail("malformed " + raw + "theta.txt");
        const size_t npix = (size_t)nimage * nimage;
        const auto p = read_u16(raw + "projections.u16", npix * nproj);
        const auto ob = read_u16(raw + "OB.u16", npix * nflat);
        std::vector<uint16_t> df;
        if (ndark > 0) df = read_u16(raw + "DF.u16", npix * ndark);
        const char* m = std::getenv("ACUMEN_NORM_MODE");
        const int mode = m ? std::atoi(m) : 0;
        std::vector<float> out(npix * nproj);
        acu_ctx* ctx = nullptr;
        check(acu_ctx_create(&ctx, 0, 0, nullptr, 0), nullptr);
        check(acu_normalize_stack_u16(ctx, mode, nproj, (long)npix, p.data(), nflat, ob.data(), ndark,
                                      ndark ? df.data() : nullptr, out.data()),
              ctx);
        acu_ctx_destroy(ctx);
        if (std::system(("mkdir -p '" + dir + "'").c_str()) != 0) throw Fail("cannot create " + dir);
        File(dir + "theta.dat", true).write(0, theta.data(), theta.size());
        const int add = nimage % 2 == 0 ? 1 : 0;
        // file-size limit of the split (the reference's 8e9 bytes; ACUMEN_FILE_BYTES overrides it)
        const char* fb = std::getenv("ACUMEN_FILE_BYTES");
        const float limit = fb ? (float)std::atof(fb) : 8.0e9f;
        const int n_files_sino = (int)std::ceil((4.0f * (float)(nimage + add) * (float)nproj * (float)nimage) / limit);
        const int n_files_rec =
            (int)std::ceil((4.0f * (float)(nimage + add) * (float)(nimage + add) * (float)nimage) / limit);
        // projections{k}.dat (:222-252).  The reference writes projection js of
        // file j at js - ceiling((j-1) r) - 1 but its readers
        // (projections_to_sinogram_hpc.F90:398) look at js - floor((j-1) r) - 1;
        // for a non-integer r the writer's offset is one too small (negative for
        // the first item), so the readers' convention is used here.
        for (int js = 1; js <= nproj; ++js) {
            const Where w = locate(js, nproj, n_files_sino);
            File fp(fnum(dir + "projections", w.file), true);
            fp.write(w.item * (long long)npix, out.data() + (size_t)(js - 1) * npix, npix);
        }
        write_fileinfo(dir, FileInfo{nproj, nimage, n_files_sino, n_files_rec});
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf(" Total write HPC projection data: %g\n", secs);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "raw_to_hpc: %s\n", e.what());
        return 1;
    }
}
