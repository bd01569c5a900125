/* tbsla/cpp/Vector.h -- drop-in for TBSLA's C vector handle
 * (src/cpp/interface/c/include/tbsla/cpp/Vector.h): a std::vector<double>
 * behind a C struct.  NULL handles give no-ops or false, as in the
 * reference (src/cpp/interface/c/matrix/Vector.cpp:13-136). */
#ifndef TBSLA_CINTERFACE_CPP_Vector
#define TBSLA_CINTERFACE_CPP_Vector

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

struct C_CPP_Vector {
  void *obj;
};
typedef struct C_CPP_Vector C_CPP_Vector_t;

C_CPP_Vector_t *C_CPP_Vector_create();
void C_CPP_Vector_destroy(C_CPP_Vector_t *v);
/* points the handle at an existing std::vector<double> (not owned) */
void C_CPP_Vector_set(C_CPP_Vector_t *v, void *obj);
/* copies the std::vector<double> at obj into the handle's vector */
void C_CPP_Vector_copy(C_CPP_Vector_t *v, void *obj);

void C_CPP_Vector_print(C_CPP_Vector_t *v);
/* n values s, s+1, ... */
void C_CPP_Vector_fill(C_CPP_Vector_t *v, int n, int s);
/* (size_t n, n doubles) at byte offset seek; write appends */
bool C_CPP_Vector_read(C_CPP_Vector_t *v, char *filename, int seek);
bool C_CPP_Vector_write(C_CPP_Vector_t *v, char *filename);

/* v1 += v2 (v1's length); v1 += v2[incr:]; v1 ++= v2 (append) */
bool C_CPP_Vector_add(C_CPP_Vector_t *v1, C_CPP_Vector_t *v2);
bool C_CPP_Vector_add_incr(C_CPP_Vector_t *v1, C_CPP_Vector_t *v2, int incr);
bool C_CPP_Vector_gather(C_CPP_Vector_t *v1, C_CPP_Vector_t *v2);

#ifdef __cplusplus
}
#endif

#endif
