/* Empty stand-in for HEALPix <pointing.h>: the harness defines pix2vec_ring and
 * nside2npix itself before including the reference headers. */
#pragma once
