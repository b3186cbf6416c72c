// C++ caller of the drop-in shim (include/nsg.hpp), written the way a user
// of nscale's HistologicalEntities API would write it, without OpenCV.
//
// usage: shim_segment <tile.bgr> <rows> <cols> <out_prefix>
// Reads a raw BGR uint8 tile, then writes
//   <out>.labels.i32   segmentNuclei(img, output, compcount, bbox) labels
//   <out>.bbox.i32     its bbox array (5 * compcount ints)
//   <out>.mask.u8      the mask overload's output
//   <out>.dlabels.i32  the device-tile overload's labels
//   <out>.rbc.u8       getRBC of the device tile
//   <out>.txt          "status compcount mask_status device_status device_compcount"
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <vector>

#include "nsg.hpp"

template <typename T>
static bool write_all(const std::string &path, const T *p, size_t n) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = fwrite(p, sizeof(T), n, f) == n;
    return fclose(f) == 0 && ok;
}

int main(int argc, char **argv) {
    if (argc != 5) {
        fprintf(stderr, "usage: %s tile.bgr rows cols out_prefix\n", argv[0]);
        return 2;
    }
    const int rows = atoi(argv[2]), cols = atoi(argv[3]);
    const std::string out = argv[4];
    nscale::HostImage<uint8_t> img(rows, cols, 3);
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(img.data(), 1, img.pixels.size(), f) != img.pixels.size()) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    fclose(f);
    try {
        nscale::HostImage<int32_t> labels;
        int compcount = 0;
        int *bbox = NULL;
        const int status = nscale::HistologicalEntities::segmentNuclei(img, labels, compcount, bbox);
        nscale::HostImage<uint8_t> mask;
        const int mstatus = nscale::HistologicalEntities::segmentNuclei(img, mask);

        nscale::DeviceImage<uint8_t> dimg = nscale::DeviceImage<uint8_t>::upload(img);
        nscale::DeviceImage<int32_t> dlabels;
        int dcount = 0;
        int *dbbox = NULL;
        const int dstatus = nscale::HistologicalEntities::segmentNuclei(dimg, dlabels, dcount, dbbox);
        const nscale::HostImage<uint8_t> rbc = nscale::HistologicalEntities::getRBC(dimg).download();

        bool ok = write_all(out + ".labels.i32", labels.data(), labels.pixels.size()) &&
                  write_all(out + ".bbox.i32", bbox ? bbox : (int *)"", bbox ? (size_t)5 * compcount : 0) &&
                  write_all(out + ".mask.u8", mask.data(), mask.pixels.size()) &&
                  write_all(out + ".dlabels.i32", dlabels.download().data(), (size_t)rows * cols) &&
                  write_all(out + ".rbc.u8", rbc.data(), rbc.pixels.size());
        free(bbox);
        free(dbbox);
        FILE *t = fopen((out + ".txt").c_str(), "w");
        if (!t) return 3;
        fprintf(t, "%d %d %d %d %d\n", status, compcount, mstatus, dstatus, dcount);
        fclose(t);
        return ok ? 0 : 3;
    } catch (const nscale::Error &e) {
        fprintf(stderr, "nscale::Error %d: %s\n", e.code(), e.what());
        return 1;
    }
}
