/* Empty stand-in for HEALPix's <healpix_map.h>: hmaps.h includes it, but the
 * map-filling template only needs pix2vec_ring, which the harness provides. */
#pragma once
