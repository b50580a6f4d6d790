/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Version and feature queries (reference: include/chromadec/version.h.in).
 * The version is the reference release this ABI mirrors. */
#ifndef CHROMADEC_VERSION_H
#define CHROMADEC_VERSION_H

#ifdef __cplusplus
extern "C" {
#endif

#define CHROMADEC_VERSION_MAJOR 0
#define CHROMADEC_VERSION_MINOR 2
#define CHROMADEC_VERSION_PATCH 1
#define CHROMADEC_VERSION_STRING "0.2.1"

const char *chd_version_string(void);
void        chd_version(int *major, int *minor, int *patch);
/* "cuda" and "gb300" answer 1; every other feature name 0. */
int         chd_has_feature(const char *feature);

#ifdef __cplusplus
}
#endif
#endif
