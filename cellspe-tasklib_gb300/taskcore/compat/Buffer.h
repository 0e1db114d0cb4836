// Stand-in for the swspectrometer's Buffer class (spectrometer/src/Buffer.h),
// used where that source tree is not on the include path.  The class keeps
// the original's members and methods in the same order, so objects created
// by a swspectrometer build and this header have the same layout; the
// methods are defined inline here (the original defines them in Buffer.cpp).
#ifndef BUFFER_H
#define BUFFER_H

#include <cstddef>
#include <cstdlib>
#include <cstring>

class Buffer
{
private:
   char* data;             // 128-byte aligned storage
   size_t len_allocated;   // bytes allocated
   size_t length;          // bytes of valid data

public:
   explicit Buffer(size_t bytes) : data(nullptr), len_allocated(bytes), length(0)
   {
      void* p = nullptr;
      if (posix_memalign(&p, 128, bytes > 0 ? bytes : 1) == 0) data = static_cast<char*>(p);
      else len_allocated = 0;
   }
   ~Buffer() { std::free(data); }
   Buffer(const Buffer&) = delete;
   Buffer& operator=(const Buffer&) = delete;

   char* getData() { return data; }
   size_t getLength() { return length; }
   size_t getAllocated() { return len_allocated; }
   void setLength(size_t len) { length = len; }
};

#endif // BUFFER_H
