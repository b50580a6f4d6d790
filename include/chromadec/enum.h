/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Drop-in declaration of the reference's public enum macro
 * (reference: include/chromadec/enum.h:1-18). C++ and C23 give every public
 * enum a fixed int32_t underlying type; older C sees a plain enum with the
 * same 4-byte representation. */
#ifndef CHROMADEC_ENUM_H
#define CHROMADEC_ENUM_H

#include <stdint.h>

#if defined(__cplusplus) || (defined(__STDC_VERSION__) && __STDC_VERSION__ >= 202311L)
#define CHD_ENUM(name) enum name : int32_t
#else
#define CHD_ENUM(name) enum name
#endif

#endif
