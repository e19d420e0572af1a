// Joints of the restatement (revolute). TEST INFRASTRUCTURE (oracle).
#include "port.h"

void p_prepare_joint( World* w, Joint* j, float h, float inv_h, Softness jointSoftness )
{
	(void)w; (void)j; (void)h; (void)inv_h; (void)jointSoftness;
}
void p_warm_start_joint( World* w, Joint* j )
{
	(void)w; (void)j;
}
void p_solve_joint( World* w, Joint* j, float h, float inv_h, int useBias )
{
	(void)w; (void)j; (void)h; (void)inv_h; (void)useBias;
}
