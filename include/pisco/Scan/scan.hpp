// Scan -- non-owning pointing view, same interface as the reference
// (src/Scan/scan.hpp:9-34): ra, dec, pa float arrays of nsamples (radians).
#ifndef PISCO_SCAN_HPP
#define PISCO_SCAN_HPP

class Scan {
  public:
    explicit Scan(long nsamples) : ra(nullptr), dec(nullptr), pa(nullptr), nsamp(nsamples) {}
    Scan(long nsamples, float* ra_, float* dec_, float* pa_)
        : ra(ra_), dec(dec_), pa(pa_), nsamp(nsamples) {}
    ~Scan() {}
    long get_nsamples(void) const { return nsamp; }
    float* get_ra_ptr(void) { return ra; }
    float* get_dec_ptr(void) { return dec; }
    float* get_pa_ptr(void) { return pa; }

  private:
    float* ra;
    float* dec;
    float* pa;
    long nsamp;
};

#endif
