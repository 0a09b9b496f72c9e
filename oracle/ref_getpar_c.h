/* Force-included ahead of the reference's param.cpp when it is built as a
 * checker (oracle/build_ref.py): the reference's getpar.cpp only compiles as
 * C, so its four entry points get C linkage here; the reference header's
 * later declarations keep that linkage. */
#ifdef __cplusplus
extern "C" {
#endif
int getpar(char *name, char *type, const void *val);
int mstpar(char *name, char *type, const void *val);
int setpar(int ac, char **av);
void endpar();
#ifdef __cplusplus
}
#endif
