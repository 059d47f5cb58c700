/* Prototype of get_python_domain (defined in the reference's
 * sw_domain_fun.h, which is compiled in the same unit after
 * shallow_water_ext.c): without it, gravity_wb's call would be an implicit
 * int declaration that conflicts with the later definition. */
struct domain;
struct _object;
struct domain *get_python_domain(struct domain *D, struct _object *domain);
