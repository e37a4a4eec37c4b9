// A stand-in for the reference's vbElphyModel<T> (electrophysiology/src/CellModel/
// ElphyModelBasis.h:184-323) for compiling the per-node view where the reference tree is absent:
// the same virtual methods with the same signatures (the interface the view must implement),
// and the base class's own backup helpers (WriteStatus / ReadStatus / Set write and read the
// GetSize() bytes at GetBase(), as the reference's kaWrite / kaRead / memcpy do on a
// little-endian 64-bit host).
#pragma once

#include <cstdio>
#include <cstring>
#include <ostream>
#include <string>
#include <vector>

template <class T>
class vbElphyModel {
 public:
  virtual ~vbElphyModel() {}
  virtual void Init(void) = 0;
  virtual void Print(std::ostream &, double, T) = 0;
  virtual void LongPrint(std::ostream &, double, T) = 0;
  virtual void GetParameterNames(std::vector<std::string> &) = 0;
  virtual void GetLongParameterNames(std::vector<std::string> &) = 0;
  virtual T GetVm(void) = 0;
  virtual T GetCai(void) = 0;
  virtual T GetCao(void) = 0;
  virtual T GetNai(void) = 0;
  virtual T GetNao(void) = 0;
  virtual T GetKi(void) = 0;
  virtual T GetKo(void) = 0;
  virtual int GetSize(void) = 0;
  virtual T *GetBase(void) = 0;
  virtual T Volume(void) = 0;
  virtual T GetAmplitude(void) = 0;
  virtual T GetStimTime(void) = 0;
  virtual T Calc(double tinc, T V, T i_external = 0., T stretch = 1., int euler = 1) = 0;
  virtual bool AddHeteroValue(std::string, double) { return false; }

  void WriteStatus(FILE *to) { std::fwrite(GetBase(), sizeof(T), (size_t)GetSize() / sizeof(T), to); }
  void ReadStatus(FILE *from) {
    if (std::fread(GetBase(), sizeof(T), (size_t)GetSize() / sizeof(T), from) != (size_t)GetSize() / sizeof(T))
      throw std::string("short read");
  }
  virtual void Set(vbElphyModel &from) { std::memcpy(GetBase(), from.GetBase(), from.GetSize()); }
};
