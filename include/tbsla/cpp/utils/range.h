/* tbsla/cpp/utils/range.h -- drop-in for TBSLA's C block split
 * (src/cpp/interface/c/include/tbsla/cpp/utils/range.h): lnv = values held
 * by part l of g parts of s values, pflv = index of its first value. */
#ifndef TBSLA_CINTERFACE_CPP_range
#define TBSLA_CINTERFACE_CPP_range

#ifdef __cplusplus
extern "C" {
#endif

static int lnv(int s, int l, int g) { return s / g + (l < s % g ? 1 : 0); }

static int pflv(int s, int l, int g) { return lnv(s, l, g) * l + (l >= s % g ? s % g : 0); }

#ifdef __cplusplus
}
#endif

#endif
