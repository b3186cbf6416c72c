// ref_cc_wrap.cpp — C entry points over the reference's own ConnComponents
// (src/segment/ConnComponents.cpp, compiled from the nscale sources by
// oracle/Makefile into oracle/_ref/).  TEST INFRASTRUCTURE ONLY: used to pin
// the oracle's CCL / area-threshold / bounding-box restatement against the
// reference implementation itself.  The reference's find()/flatten() recurse
// (ConnComponents.cpp:24-32, 137-147), so every call runs on a thread with a
// large stack.
#include "ConnComponents.h"
#include <pthread.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>

namespace {
struct Job {
    int kind;
    const unsigned char *img;
    const int *lab_in;
    int *lab_out;
    int w, h, bgval, conn, lower, upper;
    int result;
    int *bbox;
};
void *run(void *arg) {
    Job *j = (Job *)arg;
    nscale::ConnComponents cc;
    if (j->kind == 0) {
        cc.label((unsigned char *)j->img, j->w, j->h, j->lab_out, j->bgval, j->conn);
    } else if (j->kind == 1) {
        j->result = cc.areaThresholdLabeled(j->lab_in, j->w, j->h, j->lab_out, j->bgval, j->lower, j->upper);
    } else if (j->kind == 2) {
        int count = 0;
        int *b = cc.boundingBox(j->w, j->h, j->lab_in, j->bgval, count);
        j->result = count;
        if (j->bbox) memcpy(j->bbox, b, sizeof(int) * 5 * (size_t)count);
        free(b);
    } else if (j->kind == 3) {
        j->result = cc.areaThreshold((unsigned char *)j->img, j->w, j->h, j->lab_out, j->bgval, j->lower, j->upper, j->conn);
    }
    return 0;
}
int go(Job *j) {
    pthread_attr_t a;
    pthread_attr_init(&a);
    pthread_attr_setstacksize(&a, (size_t)2 << 30);
    pthread_t t;
    if (pthread_create(&t, &a, run, j) != 0) return -1;
    pthread_join(t, 0);
    pthread_attr_destroy(&a);
    return 0;
}
}  // namespace

extern "C" {
int ref_cc_label(const unsigned char *img, int w, int h, int *label, int bgval, int conn) {
    Job j = {0, img, 0, label, w, h, bgval, conn, 0, 0, 0, 0};
    return go(&j);
}
int ref_cc_area_threshold_labeled(const int *label, int w, int h, int *out, int bgval, int lower, int upper) {
    Job j = {1, 0, label, out, w, h, bgval, 0, lower, upper, 0, 0};
    if (go(&j)) return -1;
    return j.result;
}
int ref_cc_bounding_box(const int *label, int w, int h, int bgval, int *bbox_out) {
    Job j = {2, 0, label, 0, w, h, bgval, 0, 0, 0, 0, bbox_out};
    if (go(&j)) return -1;
    return j.result;
}
int ref_cc_area_threshold(const unsigned char *img, int w, int h, int *label, int bgval, int lower, int upper, int conn) {
    Job j = {3, img, 0, label, w, h, bgval, conn, lower, upper, 0, 0};
    if (go(&j)) return -1;
    return j.result;
}
}
