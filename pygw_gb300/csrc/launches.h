// Launch bookkeeping shared by the entry points (see pg_launch_count).
#pragma once
void pg_count_launches(unsigned long long n);
