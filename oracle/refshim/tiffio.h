// Stand-in for libtiff (absent here), used only to compile the reference's
// Grid.cpp for the test oracle. Grid::load_tiff is never called; every entry
// point reports failure.
#pragma once
#include <cstdint>
typedef struct tiff TIFF;
#define TIFFTAG_IMAGEWIDTH 256
#define TIFFTAG_IMAGELENGTH 257
inline TIFF* TIFFOpen(const char*, const char*) { return nullptr; }
inline void TIFFClose(TIFF*) {}
inline int TIFFGetField(TIFF*, uint32_t, ...) { return 0; }
inline int TIFFReadDirectory(TIFF*) { return 0; }
inline int TIFFSetDirectory(TIFF*, uint16_t) { return 0; }
inline int TIFFReadRGBAImage(TIFF*, uint32_t, uint32_t, uint32_t*, int = 0) { return 0; }
