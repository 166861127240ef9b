// fits_to_hpc: the drop-in for tomography/fits_to_hpc.F90 with the same
// inputs and outputs, without cfitsio or MPI.
//   inputs  $ROOT_CT_DIR/$EXP_CT_NAME/projections/*  (one FITS image each)
//           $ROOT_CT_DIR/$EXP_CT_NAME/OB/*, DF/*       (open beam, dark field)
//   outputs .../reconstruction/theta.dat, projections{k}.dat,
//           fileinfo_projections.dat
// Files are taken in name order, as the reference's `ls` (:57-97, :113-150).
// Each projection's angle comes from its name with the reference's rule
// (:75-96): the digits at 1-based positions len(EXP_CT_NAME)+11..+13 are the
// hundreds, tens and units of a degree and those at +15..+17 the tenths,
// hundredths and thousandths, accumulated in single precision; a character
// that is not a digit leaves the previous digit's value in place, as the
// reference's failed integer read does.  The grid side is NAXIS1 of the first
// open-beam image (:160-170).  Open-beam and dark frames are averaged in file
// order in single precision (:174-210); the projections are log-normalised on
// the GPU (:243, or :244 with ACUMEN_NORM_MODE=1) and written split over
// n_files_sino files of at most ~8e9 bytes (:217-252).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <dirent.h>

#include "fits.h"
#include "hpc_io.h"

static std::vector<std::string> list_files(const std::string& dir)
{
    std::vector<std::string> names;
    DIR* d = opendir(dir.c_str());
    if (!d) throw hpc::Fail("cannot list " + dir);
    while (dirent* e = readdir(d)) {
        const std::string n = e->d_name;
        if (n != "." && n != "..") names.push_back(n);
    }
    closedir(d);
    std::sort(names.begin(), names.end());   // byte order, as `ls` in the C locale
    return names;
}

// tomography/fits_to_hpc.F90:75-96
static float theta_from_name(const std::string& name, size_t exp_len, int& last_digit)
{
    const size_t p1 = exp_len + 10, p2 = exp_len + 14;   // 0-based positions of the two digit groups
    const float scale[6] = {100.0f, 10.0f, 1.0f, 0.1f, 0.01f, 0.001f};
    float th = 0.0f;
    for (int k = 0; k < 6; ++k) {
        const size_t pos = (k < 3 ? p1 : p2) + (k % 3);
        if (pos < name.size() && name[pos] >= '0' && name[pos] <= '9') last_digit = name[pos] - '0';
        th = th + scale[k] * (float)last_digit;
    }
    return th;
}

static void average(const std::string& dir, const std::vector<std::string>& files, long nimage,
                    std::vector<float>& avg)
{
    const size_t npix = (size_t)nimage * nimage;
    avg.assign(npix, 0.0f);
    for (const auto& f : files) {
        const hpc::FitsImage im = hpc::read_fits(dir + f);
        if (im.naxis1 != nimage || im.naxis2 < nimage) throw hpc::Fail(dir + f + ": not " + std::to_string(nimage) + " x " + std::to_string(nimage));
        for (size_t i = 0; i < npix; ++i) avg[i] = avg[i] + im.data[i];
    }
    const float n = (float)files.size();
    for (auto& v : avg) v = v / n;
}

int main()
{
    try {
        using namespace hpc;
        const auto t0 = std::chrono::steady_clock::now();
        const std::string exp = env("EXP_CT_NAME");
        const std::string base = env("ROOT_CT_DIR") + "/" + exp + "/", dir = base + "reconstruction/";
        const auto pnames = list_files(base + "projections/");
        const int nfiles = (int)pnames.size();
        if (nfiles < 1) throw Fail("no projections in " + base + "projections/");
        std::printf(" Number of raw projections:  %d\n", nfiles);
        std::vector<float> theta(nfiles);
        int last = 0;
        for (int j = 0; j < nfiles; ++j) theta[j] = theta_from_name(pnames[j], exp.size(), last);
        const auto obn = list_files(base + "OB/");
        const auto dfn = list_files(base + "DF/");
        std::printf(" Number of background projections:  %d\n", (int)obn.size());
        std::printf(" Number of dark field projections:  %d\n", (int)dfn.size());
        if (obn.empty()) throw Fail("no open-beam images in " + base + "OB/");
        const long nimage = read_fits(base + "OB/" + obn[0]).naxis1;
        const size_t npix = (size_t)nimage * nimage;
        std::vector<float> ob, df;
        std::printf(" Determining Average Background\n");
        average(base + "OB/", obn, nimage, ob);
        std::printf(" Determining Average Dark Field\n");
        if (!dfn.empty()) average(base + "DF/", dfn, nimage, df);
        else df.assign(npix, 0.0f);
        const char* m = std::getenv("ACUMEN_NORM_MODE");
        const int mode = m ? std::atoi(m) : 0;
        if (mode == 1 && dfn.empty()) throw Fail("ACUMEN_NORM_MODE=1 needs dark frames in " + base + "DF/");

        if (std::system(("mkdir -p '" + dir + "'").c_str()) != 0) throw Fail("cannot create " + dir);
        File(dir + "theta.dat", true).write(0, theta.data(), theta.size());
        const int add = nimage % 2 == 0 ? 1 : 0;
        const char* fb = std::getenv("ACUMEN_FILE_BYTES");
        const float limit = fb ? (float)std::atof(fb) : 8.0e9f;
        const int n_files_sino =
            (int)std::ceil((4.0f * (float)(nimage + add) * (float)nfiles * (float)nimage) / limit);
        const int n_files_rec =
            (int)std::ceil((4.0f * (float)(nimage + add) * (float)(nimage + add) * (float)nimage) / limit);

        acu_ctx* ctx = nullptr;
        check(acu_ctx_create(&ctx, 0, 0, nullptr, 0), nullptr);
        const int batch = 32;   // projections read, normalised and written together
        std::vector<float> raw(npix * batch), out(npix * batch);
        for (int j0 = 0; j0 < nfiles; j0 += batch) {
            const int nb = std::min(batch, nfiles - j0);
            for (int k = 0; k < nb; ++k) {
                const FitsImage im = read_fits(base + "projections/" + pnames[j0 + k]);
                if (im.naxis1 != nimage || im.naxis2 < nimage)
                    throw Fail(pnames[j0 + k] + ": not " + std::to_string(nimage) + " x " + std::to_string(nimage));
                std::copy(im.data.begin(), im.data.begin() + npix, raw.begin() + (size_t)k * npix);
            }
            check(acu_normalize_stack(ctx, mode, nb, (long)npix, raw.data(), ob.data(), df.data(), out.data()), ctx);
            // projections{k}.dat at the readers' offsets (see raw_to_hpc)
            for (int k = 0; k < nb; ++k) {
                const int js = j0 + k + 1;
                const Where w = locate(js, nfiles, n_files_sino);
                File fp(fnum(dir + "projections", w.file), true);
                fp.write(w.item * (long long)npix, out.data() + (size_t)k * npix, npix);
                std::printf(" Processing data %s\n", pnames[js - 1].c_str());
            }
        }
        acu_ctx_destroy(ctx);
        write_fileinfo(dir, FileInfo{nfiles, (int)nimage, n_files_sino, n_files_rec});
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf(" Total write HPC projection data: %g\n", secs);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "fits_to_hpc: %s\n", e.what());
        return 1;
    }
}
