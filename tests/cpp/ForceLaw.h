// Test stand-in for the reference's src/halo_finder/ForceLaw.h: the drop-in
// headers need only the abstract ForceLaw with its virtual f_over_r
// (ForceLaw.h:95-101).  The driver derives the laws it passes from it.
#ifndef FORCELAW_H
#define FORCELAW_H

class ForceLaw {
 public:
  ForceLaw() {}
  virtual ~ForceLaw() {}
  virtual float f_over_r(float r2) = 0;
};

#endif
