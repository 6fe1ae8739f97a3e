function mpc = m_edge
%% six buses, eight branches
mpc.version = '2';
mpc.baseMVA = 100;

%% bus data
%	bus_i	type	Pd	Qd	Gs	Bs	area	Vm	Va	baseKV	zone	Vmax	Vmin
mpc.bus = [
	10	3	0	0	0	0	1	1.02	5	230	1	1.1	0.9;
	20	2	20	10	0	0	1	1.01	0	230	1	1.1	0.9;
	30	1	45	15	0	0	1	1	0	230	1	1.1	0.9;	% a generator row names this PQ bus
	40	1	40	5	0	19	1	1	0	230	1	1.1	0.9;

	50	2	10	3	0	0	1	0.995	0	230	1	1.1	0.9;
	60	1	60	12	2	-5	1	1	0	230	1	1.1	0.9;
];

%% generator data
mpc.gen = [
	10	0	0	300	-300	1.02	100	1	300	0	0	0	0	0	0	0	0	0	0	0	0;
	20	40	0	30	-10	1.01	100	1	100	0	0	0	0	0	0	0	0	0	0	0	0;
	30	25	5	10	-10	1	100	1	50	0	0	0	0	0	0	0	0	0	0	0	0;
	50	30	0	25	-5	0.995	100	1	60	0	0	0	0	0	0	0	0	0	0	0	0;
	50	99	0	99	-99	1	100	1	99	0	0	0	0	0	0	0	0	0	0	0	0;
];

%% branch data
%	fbus	tbus	r	x	b	rateA	rateB	rateC	ratio	angle	status	angmin	angmax
mpc.branch = [
	10	20	0.01	0.06	0.05	0	0	0	0	0	1	-360	360;
	10	20	0.02	0.08	0.04	0	0	0	0	0	1	-360	360;
	20	30	0.005	0.05	0.03	0	0	0	0.97	0	1	-360	360;
% a phase shifter written with ratio 0
	30	40	0	0.04	0	0	0	0	0	-3	1	-360	360;
	40	50	0.02	0.1	0.02	0	0	0	1.03	2	1	-360	360;
	50	60	0.015	0.07	0.02	0	0	0	0	0	1	-360	360;
	60	10	0.01	0.05	0.03	0	0	0	0	0	1	-360	360;
	20	60	0.03	0.12	0.025	0	0	0	0	0	1	-360	360;
];

%% generator cost data
mpc.gencost = [
	2	0	0	3	0.01	40	0;
];
