/* SPDX-License-Identifier: GPL-3.0-or-later */
/* Umbrella header of the chd_* ABI (reference: include/chromadec/chromadec.h).
 * The NN model calls answer as a reference build without an inference
 * backend does. */
#ifndef CHROMADEC_CHROMADEC_H
#define CHROMADEC_CHROMADEC_H

#include <chromadec/version.h>
#include <chromadec/errors.h>
#include <chromadec/log.h>
#include <chromadec/types.h>
#include <chromadec/video.h>
#include <chromadec/decoder.h>
#include <chromadec/frame.h>
#include <chromadec/dropout.h>
#include <chromadec/pipeline.h>
#include <chromadec/nn.h>

#endif
