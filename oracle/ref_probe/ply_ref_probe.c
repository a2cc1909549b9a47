/* oracle/ref_probe/ply_ref_probe.c - TEST INFRASTRUCTURE ONLY. Reads a PLY file with the
 * reference's vendored rply (third_party/rply/rply/rply.c, compiled in place by
 * build_ref.py) the way the reference's readPLY does (filePLY.cpp:199-257): vertex x, y, z
 * and nx, ny, nz through read callbacks (doubles stored to floats), and the faces'
 * vertex_indices lists. Polygons are returned as read (the reference then cuts them into
 * triangles). Two calls: counts, then the data. */
#include <stdlib.h>
#include <string.h>

#include "rply.h"

typedef struct {
    float *xyz, *nrm;
    long   nv, nn;
    int   *idx, *len;
    long   nf, ni;
    int    counting;
} State;

static int vertex_cb(p_ply_argument a) {
    State *s;
    long   axis;
    ply_get_argument_user_data(a, (void **)&s, &axis);
    if (!s->counting)
        s->xyz[3 * s->nv + axis] = (float)ply_get_argument_value(a);
    if (axis == 2)
        s->nv++;
    return 1;
}

static int normal_cb(p_ply_argument a) {
    State *s;
    long   axis;
    ply_get_argument_user_data(a, (void **)&s, &axis);
    if (!s->counting)
        s->nrm[3 * s->nn + axis] = (float)ply_get_argument_value(a);
    if (axis == 2)
        s->nn++;
    return 1;
}

static int face_cb(p_ply_argument a) {
    State *s;
    long   dummy, length, index;
    ply_get_argument_user_data(a, (void **)&s, &dummy);
    ply_get_argument_property(a, NULL, &length, &index);
    if (index == -1) {
        if (!s->counting)
            s->len[s->nf] = (int)length;
        s->nf++;
        return 1;
    }
    if (!s->counting)
        s->idx[s->ni] = (int)ply_get_argument_value(a);
    s->ni++;
    return 1;
}

static int run(const char *path, State *s) {
    p_ply ply = ply_open(path, NULL, 0, NULL);
    if (!ply)
        return 1;
    if (!ply_read_header(ply)) {
        ply_close(ply);
        return 2;
    }
    ply_set_read_cb(ply, "vertex", "x", vertex_cb, s, 0);
    ply_set_read_cb(ply, "vertex", "y", vertex_cb, s, 1);
    ply_set_read_cb(ply, "vertex", "z", vertex_cb, s, 2);
    ply_set_read_cb(ply, "vertex", "nx", normal_cb, s, 0);
    ply_set_read_cb(ply, "vertex", "ny", normal_cb, s, 1);
    ply_set_read_cb(ply, "vertex", "nz", normal_cb, s, 2);
    ply_set_read_cb(ply, "face", "vertex_indices", face_cb, s, 0);
    const int ok = ply_read(ply);
    ply_close(ply);
    return ok ? 0 : 3;
}

/* counts[4] = {vertices, normals, faces, face indices} */
int ref_ply_counts(const char *path, long *counts) {
    State s;
    memset(&s, 0, sizeof(s));
    s.counting = 1;
    const int r = run(path, &s);
    counts[0] = s.nv;
    counts[1] = s.nn;
    counts[2] = s.nf;
    counts[3] = s.ni;
    return r;
}

int ref_ply_read(const char *path, float *xyz, float *nrm, int *len, int *idx) {
    State s;
    memset(&s, 0, sizeof(s));
    s.xyz = xyz;
    s.nrm = nrm;
    s.len = len;
    s.idx = idx;
    return run(path, &s);
}
