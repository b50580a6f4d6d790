/* A C11 consumer written against the chd_* headers only, the way a program
 * built for the reference uses the library (tests/unit/abi_smoke.c and
 * test_integration.cpp:277-330 in the reference follow the same calls).
 * Linked with -lchromadec, i.e. by the reference's library name.
 *
 *   consumer <capture.tbc> [decode]
 *
 * Prints one line of JSON: version, video info, output info and the dropout
 * spans of frame 0; with "decode", also the first Y/Cb/Cr samples of frame 0
 * decoded with CHD_DEC_TRANSFORM_3D. */
#include <chromadec/chromadec.h>

#include <stdio.h>
#include <string.h>

#define CHECK(call)                                                                            \
    do {                                                                                       \
        chd_status_t s_ = (call);                                                              \
        if (s_ != CHD_OK) {                                                                    \
            printf("{\"error\": \"%s\", \"status\": \"%s\", \"detail\": \"%s\"}\n", #call,   \
                   chd_status_str(s_), chd_last_error());                                      \
            return 1;                                                                          \
        }                                                                                      \
    } while (0)

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    CHECK(chd_init());
    chd_video_t *v = NULL;
    CHECK(chd_video_open_composite(argv[1], NULL, NULL, &v));
    chd_video_info_t vi;
    CHECK(chd_video_get_info(v, &vi));

    chd_decoder_t *d = NULL;
    CHECK(chd_decoder_create(v, CHD_DEC_NONE, &d));
    CHECK(chd_decoder_set_option_i32(d, CHD_OPT_PADDING_MULTIPLE, 1));
    CHECK(chd_decoder_commit(d));
    chd_output_info_t oi;
    CHECK(chd_decoder_get_output_info(d, &oi));
    chd_dropout_span_t *spans = NULL;
    size_t n = 0;
    CHECK(chd_decoder_get_dropout_spans(d, 0, CHD_DROPOUT_DETECTED, &spans, &n));

    printf("{\"version\": \"%s\", \"field_width\": %d, \"num_frames\": %lld, \"out\": [%d, %d, %d], \"spans\": [",
           chd_version_string(), vi.field_width, (long long)vi.num_frames, oi.width, oi.height, oi.num_planes);
    for (size_t i = 0; i < n; i++)
        printf("%s[%d, %d, %d, %d]", i ? ", " : "", spans[i].y, spans[i].x_start, spans[i].x_end, (int)spans[i].origin);
    printf("]");
    chd_dropout_spans_free(spans);
    chd_decoder_free(d);

    if (argc > 2 && strcmp(argv[2], "decode") == 0) {
        chd_decoder_t *t = NULL;
        CHECK(chd_decoder_create(v, CHD_DEC_TRANSFORM_3D, &t));
        CHECK(chd_decoder_set_option_str(t, CHD_OPT_OUTPUT_FORMAT, "yuv444p16"));
        CHECK(chd_decoder_commit(t));
        chd_frame_t *f = NULL;
        CHECK(chd_decode_frame(t, 0, &f));
        chd_frame_info_t fi;
        CHECK(chd_frame_get_info(f, &fi));
        printf(", \"frame\": [%d, %d, %d], \"samples\": [", fi.width, fi.height, fi.num_planes);
        for (int p = 0; p < 3; p++) {
            const void *data = NULL;
            ptrdiff_t stride = 0;
            CHECK(chd_frame_get_plane(f, (chd_plane_t)p, &data, &stride));
            const uint16_t *row = (const uint16_t *)((const char *)data + 300 * stride);
            printf("%s%u", p ? ", " : "", row[474]);
        }
        printf("]");
        chd_frame_free(f);
        chd_decoder_free(t);
    }
    printf("}\n");
    chd_video_free(v);
    chd_shutdown();
    return 0;
}
